// Differentiation of the AdResS step: a hand-written adjoint (reverse mode)
// of the weighted LJ pair force of LJ_IdealGas (LJ_IdealGas.cpp:52-225, with
// the drift force -V_ij grad lambda and the compensation force), of the
// thermodynamic force (ThermodynamicForce.hpp:98-122) and of the Langevin
// velocity-Verlet step (VelocityVerletLangevinThermostat.hpp:48-121,
// VelocityVerlet.cpp:69-90), on top of the batched replica engine.
//
// The loss is the squared deviation from uniform of the Gaussian-smoothed
// x-density profile averaged over the last `window` steps of a trajectory
// of `steps` steps.  Its gradient with respect to the thermodynamic-force
// table and to the LJ epsilon and sigma is computed by the adjoint sweep:
// the forward run stores a checkpoint every `checkpointInterval` steps; the
// backward sweep recomputes each segment from its checkpoint, keeps the
// pre-force positions of every step of the segment and runs the adjoint
// steps backwards.  Neighbour list, ghosts, the force cap branch, cutoff and
// TF bins are piecewise constant: the adjoint is the derivative almost
// everywhere.  The drift-compensation means are held fixed (compFrozen) and
// the TF table is not updated inside the trajectory, so that the table and
// epsilon/sigma are the only parameters.
//
// Force on molecule i (single site; g = grad lambda~ = (m'(x), 0, 0), m the
// modulated weight of the Slab):
//   F_i = sum_j [ w_ij f(s_ij) r_ij - e(s_ij)/2 g_i ] + mu(bin(lambda_i)) g_i + T(x_i) e_x,
//   w_ij = (m_i + m_j)/2,  r_ij = x_i - x_j,  s = |r|^2.
// With a = dL/dF (per molecule) and Phi = sum_i a_i.F_i, every unordered pair
// contributes w f (da.r) - e/2 (a_i.g_i + a_j.g_j), da = a_i - a_j, so
//   dPhi/dx_i = sum_j [ g_i/2 f q + w (2 f' q r + f da) - e' r (a_i.g_i + a_j.g_j) ]
//               - (sum_j e)/2 a_ix m''_i e_x + mu a_ix m''_i e_x,    q = da.r,
// and dPhi/dtheta = sum_pairs [ w q df/dtheta - de/dtheta (a_i.g_i + a_j.g_j)/2 ].
// The full list visits every pair from both sides, so each row writes its
// own dPhi/dx_i (no scatter) and adds half of the parameter terms.
#include <cmath>
#include <cstring>
#include <vector>

#include "batch_impl.cuh"

using namespace mrmd_impl;
using namespace mrmd_batch_impl;

namespace
{
// LJ parameters and their derivatives with respect to epsilon and sigma
// (constructor and precompute of action/LennardJones.cpp).
struct LJDiff
{
    double eps, rcSqr, capSqr, rcap;
    double ff1, ff2, ef1, ef2, shift, C, Ec;     // forceFactor / energy factors, cap coefficient, E(r_cap)
    double ff1s, ff2s, ef1s, ef2s;               // d/dsigma of the factors (each is proportional to epsilon)
    double Cs, Ecs, shifts;                      // d/dsigma of the cap and shift terms
};

LJDiff make_ljdiff(double eps, double sig, double rc, double rcap, int shifted)
{
    LJDiff L{};
    const double s2 = sig * sig, s6 = s2 * s2 * s2, s12 = s6 * s6;
    L.eps = eps;
    L.rcSqr = rc * rc;
    L.rcap = rcap;
    L.capSqr = rcap * rcap;
    L.ff1 = 48.0 * eps * s12;
    L.ff2 = 24.0 * eps * s6;
    L.ef1 = 4.0 * eps * s12;
    L.ef2 = 4.0 * eps * s6;
    L.ff1s = 12.0 * L.ff1 / sig;
    L.ff2s = 6.0 * L.ff2 / sig;
    L.ef1s = 12.0 * L.ef1 / sig;
    L.ef2s = 6.0 * L.ef2 / sig;
    if (rcap > 0.0)
    {
        const double u = 1.0 / L.capSqr, u3 = u * u * u;
        L.C = u3 * u * (L.ff1 * u3 - L.ff2) * rcap;
        L.Cs = u3 * u * (L.ff1s * u3 - L.ff2s) * rcap;
        L.Ec = u3 * (L.ef1 * u3 - L.ef2);
        L.Ecs = u3 * (L.ef1s * u3 - L.ef2s);
    }
    if (shifted)
    {
        const double u = 1.0 / L.rcSqr, u3 = u * u * u;
        L.shift = u3 * (L.ef1 * u3 - L.ef2);
        L.shifts = u3 * (L.ef1s * u3 - L.ef2s);
    }
    return L;
}

// f (force factor), e (energy), their s-derivatives and parameter partials
struct LJVals
{
    double f, fp, e, ep, fe, fs, ee, es;
};

__device__ __forceinline__ LJVals lj_diff(const LJDiff& L, double s)
{
    LJVals o;
    if (s >= L.capSqr)
    {
        const double u = 1.0 / s, u3 = u * u * u, u6 = u3 * u3;
        o.f = u3 * u * (L.ff1 * u3 - L.ff2);
        o.fp = u * u * (-7.0 * L.ff1 * u6 + 4.0 * L.ff2 * u3);
        o.e = u3 * (L.ef1 * u3 - L.ef2) - L.shift;
        o.ep = u * (-6.0 * L.ef1 * u6 + 3.0 * L.ef2 * u3);
        o.fs = u3 * u * (L.ff1s * u3 - L.ff2s);
        o.es = u3 * (L.ef1s * u3 - L.ef2s) - L.shifts;
    }
    else
    {
        // inside the cap: f = C / r, e = E(r_cap) - (r - r_cap) C - shift
        const double r = sqrt(s);
        o.f = L.C / r;
        o.fp = -0.5 * L.C / (s * r);
        o.e = L.Ec - (r - L.rcap) * L.C - L.shift;
        o.ep = -0.5 * L.C / r;
        o.fs = L.Cs / r;
        o.es = L.Ecs - (r - L.rcap) * L.Cs - L.shifts;
    }
    // every factor is proportional to epsilon
    o.fe = o.f / L.eps;
    o.ee = o.e / L.eps;
    return o;
}

// second derivative of the modulated weight of the Slab in x
// (m = cos^n(k(|dx| - a)), m' as in Slab.hpp:96-120)
__device__ __forceinline__ double slab_m2(const SlabDev& s, double x)
{
    const double ad = fabs(x - s.cx);
    if (s.abrupt || ad < s.atHalf || ad > s.atHalf + s.hy) return 0.0;
    const double pi = 3.141592653589793238462643383279502884;
    const double k = pi / (2.0 * s.hy);
    const double u = k * (ad - s.atHalf);
    const double c = cos(u), sn = sin(u);
    const double n = (double)s.exponent;
    return -n * k * k * (pow_int(c, s.exponent) - (n - 1.0) * sn * sn * pow_int(c, s.exponent - 2));
}

// The FP32 copies of the LJDiff factors used for pairs beyond r_split in the
// mixed form (the pair force and its derivatives are small there: at most
// |F(r_split)| = 1.67 epsilon/sigma at 1.4 sigma).
struct LJDiffF
{
    float ff1, ff2, ef1, ef2, shift, ff1s, ff2s, ef1s, ef2s, shifts, invEps, rcSq;
};

LJDiffF to_float(const LJDiff& L)
{
    return LJDiffF{(float)L.ff1, (float)L.ff2, (float)L.ef1, (float)L.ef2, (float)L.shift, (float)L.ff1s,
                   (float)L.ff2s, (float)L.ef1s, (float)L.ef2s, (float)L.shifts, (float)(1.0 / L.eps),
                   (float)L.rcSqr};
}

constexpr int ADJ_TPR = 4;  // lanes per row of the adjoint pair kernel

struct AdjArgs
{
    const double4* a;  // [N] dL/dF of the step
    const float4* af;  // [N] mixed form: (a.x, a.y, a.z, a.x m') in FP32
    double4* xbar;     // [N] dL/dx, accumulated
    double* grad;      // [2] epsilon, sigma
    double* tfGrad;    // [sum bins]
    LJDiff L;
    LJDiffF Lf;
};

// dPhi/dx_i (added to xbar) and the parameter terms of one force evaluation.
// MIXED: pairs at r >= r_split are evaluated in FP32 on the split
// coordinates with FP32 sums per row; closer pairs, and pairs within the
// FP32 error band of rc, in FP64.
// TPR lanes share a row (entries k = sub, sub + TPR, ...) and reduce with a
// fixed butterfly, so that the few long rows of the atomistic and hybrid
// regions are spread over more warps.
template <bool MIXED, int TPR>
__global__ void __launch_bounds__(TB) k_adj_force(BDev B, AdjArgs A)
{
    __shared__ double red[64];
    double ge = 0.0, gs = 0.0;
    const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool valid = gtid < (int64_t)B.N * TPR;
    const int sub = (int)(gtid % TPR);
    {
        const int32_t i = valid ? (int32_t)(gtid / TPR) : 0;
        const RepDev& R = B.reps[B.slotRep[i]];
        const double4 la = B.lam[i];  // lambda, m, m'
        const double4 pi = B.pos[i];
        const double4 ai = A.a[i];
        const double agi = ai.x * la.z;
        double bx = 0.0, by = 0.0, bz = 0.0, esum = 0.0;
        float fbx = 0.f, fby = 0.f, fbz = 0.f, fesum = 0.f, fge = 0.f, fgs = 0.f;
        float4 hi_i, lo_i, afi;
        float mi = 0.f, gi = 0.f;
        if (MIXED)
        {
            hi_i = B.hi[i];
            lo_i = B.lo[i];
            afi = A.af[i];
            mi = B.lamtf[i].x;
            gi = (float)la.z;
        }
        const int cnt = valid ? B.counts[i] : 0;
        const int64_t rowBase = mrmd_dev::nbr_row(i, B.listCap);
        for (int k = sub; k < cnt; k += TPR)
        {
            const int32_t j = B.nbrs[rowBase + 32 * (int64_t)k] & 0x7fffffff;
            if (MIXED)
            {
                // no FP64 operation on the FP32 path: weights and adjoint in FP32
                const float mj = B.lamtf[j].x;
                if (mi <= 0.0f && mj <= 0.0f) continue;  // both coarse grained
                const float4 hj = B.hi[j], loj = B.lo[j];
                const float rx = (hi_i.x - hj.x) + (lo_i.x - loj.x);
                const float ry = (hi_i.y - hj.y) + (lo_i.y - loj.y);
                const float rz = (hi_i.z - hj.z) + (lo_i.z - loj.z);
                const float s = __fmaf_rn(rx, rx, __fmaf_rn(ry, ry, rz * rz));
                const LJDiffF& L = A.Lf;
                if (s > L.rcSq * 1.0000005f) continue;
                if (s >= B.rsplitSq && s < L.rcSq * 0.9999995f)
                {
                    // a ghost takes its source's adjoint and (the replica is
                    // consistent) its source's weight derivative
                    const int32_t src = j < B.N ? j : B.gSrc[j - B.N];
                    const float4 afj = A.af[src];
                    const float u = __fdividef(1.0f, s), u3 = u * u * u, u6 = u3 * u3;
                    const float f = u3 * u * __fmaf_rn(L.ff1, u3, -L.ff2);
                    const float fp = u * u * __fmaf_rn(-7.0f * L.ff1, u6, 4.0f * L.ff2 * u3);
                    const float e = __fmaf_rn(u3, __fmaf_rn(L.ef1, u3, -L.ef2), -L.shift);
                    const float ep = u * __fmaf_rn(-6.0f * L.ef1, u6, 3.0f * L.ef2 * u3);
                    const float fs = u3 * u * __fmaf_rn(L.ff1s, u3, -L.ff2s);
                    const float es = __fmaf_rn(u3, __fmaf_rn(L.ef1s, u3, -L.ef2s), -L.shifts);
                    const float w = 0.5f * (mi + mj);
                    const float dax = afi.x - afj.x, day = afi.y - afj.y, daz = afi.z - afj.z;
                    const float q = __fmaf_rn(dax, rx, __fmaf_rn(day, ry, daz * rz));
                    const float agsum = afi.w + afj.w;
                    const float c1 = 2.0f * w * fp * q - ep * agsum;
                    fbx += c1 * rx + w * f * dax + 0.5f * gi * f * q;
                    fby += c1 * ry + w * f * day;
                    fbz += c1 * rz + w * f * daz;
                    fesum += e;
                    fge += 0.5f * (w * q * f - 0.5f * e * agsum) * L.invEps;
                    fgs += 0.5f * (w * q * fs - 0.5f * es * agsum);
                    continue;
                }
            }
            const double4 lj = B.lam[j];
            if (!MIXED && la.y <= 0.0 && lj.y <= 0.0) continue;  // both coarse grained
            const double4 pj = B.pos[j];
            const double rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
            const double s = rx * rx + ry * ry + rz * rz;
            if (s > A.L.rcSqr) continue;
            const int32_t src = j < B.N ? j : B.gSrc[j - B.N];
            const double4 aj = A.a[src];
            const LJVals V = lj_diff(A.L, s);
            const double w = 0.5 * (la.y + lj.y);
            const double dax = ai.x - aj.x, day = ai.y - aj.y, daz = ai.z - aj.z;
            const double q = dax * rx + day * ry + daz * rz;
            const double agj = aj.x * lj.z;
            const double c1 = 2.0 * w * V.fp * q - V.ep * (agi + agj);
            bx += c1 * rx + w * V.f * dax + 0.5 * la.z * V.f * q;
            by += c1 * ry + w * V.f * day;
            bz += c1 * rz + w * V.f * daz;
            esum += V.e;
            ge += 0.5 * (w * q * V.fe - 0.5 * V.ee * (agi + agj));
            gs += 0.5 * (w * q * V.fs - 0.5 * V.es * (agi + agj));
        }
        if (MIXED)
        {
            bx += (double)fbx;
            by += (double)fby;
            bz += (double)fbz;
            esum += (double)fesum;
            ge += (double)fge;
            gs += (double)fgs;
        }
#pragma unroll
        for (int off = 1; off < TPR; off <<= 1)
        {
            bx += __shfl_xor_sync(0xffffffffu, bx, off);
            by += __shfl_xor_sync(0xffffffffu, by, off);
            bz += __shfl_xor_sync(0xffffffffu, bz, off);
            esum += __shfl_xor_sync(0xffffffffu, esum, off);
        }
        if (valid && sub == 0)
        {
            // curvature of the own weight: drift (-e/2 m') and compensation (mu m')
            if (is_hy(la.y))
            {
                const double m2 = slab_m2(R.slab, pi.x);
                double mu = 0.0;
                const int b = comp_bin(la.x);
                if (b != -1) mu = B.compMean[B.slotRep[i] * COMP_BINS + b];
                bx += (mu - 0.5 * esum) * ai.x * m2;
            }
            double4 xb = A.xbar[i];
            xb.x += bx;
            xb.y += by;
            xb.z += bz;
            A.xbar[i] = xb;
            if (B.tfEnabled)
            {
                const int64_t b = (int64_t)floor((pi.x - R.tfMin) * R.tfInvBin);
                if (b >= 0 && b < R.tfBins) atomicAdd(A.tfGrad + R.tfBase + b, ai.x);
            }
        }
    }
    mrmd_dev::block_sum2(ge, gs, red);
    if (threadIdx.x == 0)
    {
        atomicAdd(A.grad + 0, ge);
        atomicAdd(A.grad + 1, gs);
    }
}

// a = Fbar + h vbar: the adjoint of the step's force (it feeds the post kick
// v3 = v2 + h F and, through Fbar, the next step's pre kick)
__global__ void k_adj_prepare(const double4* __restrict__ Fbar, const double4* __restrict__ vbar,
                              double4* __restrict__ a, int32_t n, double h)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const double4 f = Fbar[i], v = vbar[i];
        a[i] = make_double4(f.x + h * v.x, f.y + h * v.y, f.z + h * v.z, 0.0);
    }
}

// FP32 copy of the adjoint for the mixed form's FP32 pair path: (a, a.x m')
__global__ void k_adj_float(const double4* __restrict__ a, const double4* __restrict__ lam, int32_t n,
                            float4* __restrict__ af)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const double4 v = a[i];
        af[i] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)(v.x * lam[i].z));
    }
}

// backwards through v1 = v + h F, x1 = x + dt/2 v1, v2 = c1 v1 + c2 xi,
// x2 = x1 + dt/2 v2, v3 = v2 + h F'(x2):  xbar holds dL/dx2 (force and loss
// terms included), vbar dL/dv3
__global__ void k_adj_vv(double4* __restrict__ xbar, double4* __restrict__ vbar, double4* __restrict__ Fbar,
                         int32_t n, double halfDt, double c1, double h)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const double4 x = xbar[i], v3 = vbar[i];
        const double v2x = v3.x + halfDt * x.x, v2y = v3.y + halfDt * x.y, v2z = v3.z + halfDt * x.z;
        const double v1x = c1 * v2x + halfDt * x.x, v1y = c1 * v2y + halfDt * x.y, v1z = c1 * v2z + halfDt * x.z;
        vbar[i] = make_double4(v1x, v1y, v1z, 0.0);
        Fbar[i] = make_double4(h * v1x, h * v1y, h * v1z, 0.0);
    }
}

// Gaussian-smoothed x-density on `bins` bin centres (periodic in x)
struct LossDev
{
    double xmin, Lx, binW, invSig2, norm, cutoff;
    int32_t bins;
    double* rho;        // [bins] sum of kernel values
    const double* coef; // [bins] dL/d(rho_b) / (window * area)
};

__global__ void k_loss_density(BDev B, LossDev D)
{
    const int span = (int)ceil(D.cutoff / D.binW) + 1;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B.N; i += gridDim.x * blockDim.x)
    {
        const double x = B.pos[i].x;
        const int b0 = (int)floor((x - D.xmin) / D.binW);
        for (int o = -span; o <= span; ++o)
        {
            int b = (b0 + o) % D.bins;
            if (b < 0) b += D.bins;
            double d = x - (D.xmin + ((double)b + 0.5) * D.binW);
            d -= D.Lx * rint(d / D.Lx);
            if (fabs(d) > D.cutoff) continue;
            atomicAdd(D.rho + b, D.norm * exp(-0.5 * d * d * D.invSig2));
        }
    }
}

__global__ void k_loss_grad(BDev B, LossDev D, double4* __restrict__ xbar)
{
    const int span = (int)ceil(D.cutoff / D.binW) + 1;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B.N; i += gridDim.x * blockDim.x)
    {
        const double x = B.pos[i].x;
        const int b0 = (int)floor((x - D.xmin) / D.binW);
        double g = 0.0;
        for (int o = -span; o <= span; ++o)
        {
            int b = (b0 + o) % D.bins;
            if (b < 0) b += D.bins;
            double d = x - (D.xmin + ((double)b + 0.5) * D.binW);
            d -= D.Lx * rint(d / D.Lx);
            if (fabs(d) > D.cutoff) continue;
            g += D.coef[b] * (-d * D.invSig2) * D.norm * exp(-0.5 * d * d * D.invSig2);
        }
        xbar[i].x += g;
    }
}
}  // namespace

struct mrmd_diff
{
    mrmd_batch* b = nullptr;
    mrmd_diff_config dc{};
    double rc = 0, rcap = 0, eps = 1, sig = 1;
    int shifted = 1;
    double area = 0, Lx = 0, xmin = 0;
    int32_t nBins = 0;  // TF table bins
    mrmd_batch_impl::Snap init;
    std::vector<mrmd_batch_impl::Snap> ckpt;
    double4* x2 = nullptr;  // [checkpointInterval][N] pre-force positions of a segment
    double4 *xbar = nullptr, *vbar = nullptr, *Fbar = nullptr, *adj = nullptr;
    float4* adjf = nullptr;  // mixed form: FP32 copy of adj
    double* grad = nullptr;    // [2]
    double* tfGrad = nullptr;  // [nBins]
    double* rho = nullptr;     // [lossBins]
    double* coef = nullptr;    // [lossBins]
    std::vector<double> hRho;
    bool haveForward = false;
};

namespace
{
LossDev loss_dev(const mrmd_diff* d)
{
    LossDev D{};
    D.xmin = d->xmin;
    D.Lx = d->Lx;
    D.bins = (int32_t)d->dc.lossBins;
    D.binW = d->Lx / (double)d->dc.lossBins;
    D.invSig2 = 1.0 / (d->dc.lossSigma * d->dc.lossSigma);
    D.norm = 1.0 / (std::sqrt(2.0 * 3.141592653589793238462643383279502884) * d->dc.lossSigma);
    D.cutoff = 6.0 * d->dc.lossSigma;
    D.rho = d->rho;
    D.coef = d->coef;
    return D;
}

// new epsilon/sigma (LJ table of the forward kernels) and TF table
int set_params(mrmd_ctx* ctx, mrmd_diff* d, const double* table, double eps, double sig)
{
    mrmd_batch* b = d->b;
    mrmd_lj_params t{};
    const double c = d->rcap, r = d->rc;
    lj_table_host(&t, 1, &c, &r, &sig, &eps, d->shifted);
    b->B.lj = to_dev(t);
    d->eps = eps;
    d->sig = sig;
    if (table) MRMD_TRY(h2d(ctx, b->B.tfForce, table, sizeof(double) * (size_t)d->nBins));
    drop_graph(b);
    return MRMD_OK;
}

int restore_initial(mrmd_ctx* ctx, mrmd_diff* d)
{
    MRMD_TRY(snapshot(ctx, d->b, d->init, false));
    d->b->steps = 0;
    d->b->needRebuild = true;
    return refresh_step_flags(ctx, d->b);
}

int accumulate_density(mrmd_ctx* ctx, mrmd_diff* d)
{
    k_loss_density<<<grid_for(ctx, d->b->N, TB), TB, 0, ctx->stream>>>(d->b->B, loss_dev(d));
    return after_launch(ctx, "loss density");
}
}  // namespace

extern "C" {

int mrmd_diff_create(mrmd_ctx* ctx, mrmd_diff** out, const mrmd_batch_config* cfg, const mrmd_replica_desc* rep,
                     const double* pos3, const double* vel3, const mrmd_diff_config* dc)
{
    if (!ctx || !out || !cfg || !rep || !pos3 || !vel3 || !dc) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(dc->steps >= 1 && dc->window >= 1 && dc->window <= dc->steps && dc->checkpointInterval >= 1 &&
                       dc->lossBins >= 2 && dc->lossSigma > 0.0,
                   ctx, "bad differentiation config");
    MRMD_CHECK_ARG(cfg->tfEnabled, ctx, "the thermodynamic force must be enabled");
    MRMD_CHECK_ARG(dc->checkpointInterval % cfg->tuning.rebuildInterval == 0, ctx,
                   "the checkpoint interval must be a multiple of the rebuild interval");
    mrmd_batch_config c = *cfg;
    c.compFrozen = 1;                       // compensation means are constants of the trajectory
    c.tfUpdateInterval = dc->steps + 1;      // the table is a parameter, not updated inside
    c.tuning.graphSteps = 0;
    c.tuning.sortEvery = 0;
    c.tuning.listLayout = 0;                 // the adjoint walks one full row per molecule
    *out = nullptr;
    mrmd_diff* d = new mrmd_diff();
    d->dc = *dc;
    d->rc = cfg->rc;
    d->rcap = cfg->cappingDistance;
    d->eps = cfg->epsilon;
    d->sig = cfg->sigma;
    d->shifted = cfg->shifted;
    d->xmin = rep->boxMin[0];
    d->Lx = rep->boxMax[0] - rep->boxMin[0];
    d->area = (rep->boxMax[1] - rep->boxMin[1]) * (rep->boxMax[2] - rep->boxMin[2]);
    int rc = mrmd_batch_create(ctx, &d->b, &c, 1, rep, pos3, vel3);
    if (rc == MRMD_OK && !d->b->reps[0].consistent)
        rc = set_error(ctx, MRMD_ERR_ARG, "differentiation needs a slab that stays clear of the ghost layer");
    const int64_t N = rc == MRMD_OK ? d->b->N : 0;
    if (rc == MRMD_OK)
    {
        d->nBins = d->b->reps[0].tfBins;
        const int64_t segs = (dc->steps + dc->checkpointInterval - 1) / dc->checkpointInterval;
        d->ckpt.resize((size_t)segs);
        rc = snap_alloc(ctx, d->b, d->init);
        for (auto& s : d->ckpt)
            if (rc == MRMD_OK) rc = snap_alloc(ctx, d->b, s);
    }
    if (rc == MRMD_OK) rc = grow(ctx, d->x2, 0, dc->checkpointInterval * N);
    if (rc == MRMD_OK) rc = grow(ctx, d->xbar, 0, N);
    if (rc == MRMD_OK) rc = grow(ctx, d->vbar, 0, N);
    if (rc == MRMD_OK) rc = grow(ctx, d->Fbar, 0, N);
    if (rc == MRMD_OK) rc = grow(ctx, d->adj, 0, N);
    if (rc == MRMD_OK) rc = grow(ctx, d->adjf, 0, N);
    if (rc == MRMD_OK) rc = grow(ctx, d->grad, 0, (int64_t)2);
    if (rc == MRMD_OK) rc = grow(ctx, d->tfGrad, 0, (int64_t)std::max(d->nBins, 1));
    if (rc == MRMD_OK) rc = grow(ctx, d->rho, 0, dc->lossBins);
    if (rc == MRMD_OK) rc = grow(ctx, d->coef, 0, dc->lossBins);
    if (rc == MRMD_OK) rc = snapshot(ctx, d->b, d->init, true);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "diff create");
    if (rc != MRMD_OK)
    {
        mrmd_diff_destroy(ctx, d);
        return rc;
    }
    d->hRho.resize((size_t)dc->lossBins);
    *out = d;
    return MRMD_OK;
}

int mrmd_diff_destroy(mrmd_ctx* ctx, mrmd_diff* d)
{
    if (!d) return MRMD_OK;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    snap_free(d->init);
    for (auto& s : d->ckpt) snap_free(s);
    void* ptrs[] = {d->x2, d->xbar, d->vbar, d->Fbar, d->adj, d->adjf, d->grad, d->tfGrad, d->rho, d->coef};
    for (void* p : ptrs) dfree(p);
    if (d->b) mrmd_batch_destroy(ctx, d->b);
    delete d;
    return MRMD_OK;
}

int mrmd_diff_num_bins(const mrmd_diff* d, int64_t* tfBins)
{
    if (!d || !tfBins) return MRMD_ERR_ARG;
    *tfBins = d->nBins;
    return MRMD_OK;
}

int mrmd_diff_set_state(mrmd_ctx* ctx, mrmd_diff* d, const double* pos3, const double* vel3)
{
    if (!ctx || !d || !pos3 || !vel3) return MRMD_ERR_ARG;
    mrmd_batch* b = d->b;
    const size_t N = (size_t)b->N;
    std::vector<double4> p(N), v(N), z(N, make_double4(0.0, 0.0, 0.0, 0.0));
    for (size_t i = 0; i < N; ++i)
    {
        p[i] = make_double4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], 0.0);
        v[i] = make_double4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.0);
    }
    MRMD_TRY(h2d(ctx, d->init.pos, p.data(), sizeof(double4) * N));
    MRMD_TRY(h2d(ctx, d->init.vel, v.data(), sizeof(double4) * N));
    MRMD_TRY(h2d(ctx, d->init.force, z.data(), sizeof(double4) * N));
    d->haveForward = false;
    return MRMD_OK;
}

int mrmd_diff_forward(mrmd_ctx* ctx, mrmd_diff* d, const double* tfTable, double epsilon, double sigma, double* loss)
{
    if (!ctx || !d || !(epsilon > 0.0) || !(sigma > 0.0)) return MRMD_ERR_ARG;
    mrmd_batch* b = d->b;
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    // the initial state first: its snapshot holds a TF table too
    int rc = restore_initial(ctx, d);
    if (rc == MRMD_OK) rc = set_params(ctx, d, tfTable, epsilon, sigma);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMemsetAsync(d->rho, 0, sizeof(double) * d->dc.lossBins, ctx->stream), "rho");
    const int64_t S = d->dc.steps, C = d->dc.checkpointInterval, W = d->dc.window;
    for (int64_t st = 0; st < S && rc == MRMD_OK; ++st)
    {
        if (st % C == 0) rc = snapshot(ctx, b, d->ckpt[(size_t)(st / C)], true);
        if (rc == MRMD_OK) rc = step(ctx, b, st, true);
        if (rc == MRMD_OK && st >= S - W) rc = accumulate_density(ctx, d);
    }
    b->steps = S;
    if (rc == MRMD_OK) rc = d2h(ctx, d->hRho.data(), d->rho, sizeof(double) * d->dc.lossBins);
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    // L = sum_b (rho_b - rho_uniform)^2, rho_b = kernel sum / (window * area)
    const double scale = 1.0 / ((double)W * d->area);
    const double uniform = (double)b->N / (d->Lx * d->area);
    double L = 0.0;
    for (double r : d->hRho)
    {
        const double dv = r * scale - uniform;
        L += dv * dv;
    }
    if (loss) *loss = L;
    d->haveForward = true;
    return MRMD_OK;
}

int mrmd_diff_backward(mrmd_ctx* ctx, mrmd_diff* d, double* gradTable, double* gradEpsilon, double* gradSigma)
{
    if (!ctx || !d) return MRMD_ERR_ARG;
    if (!d->haveForward) return set_error(ctx, MRMD_ERR_STATE, "backward needs a forward run");
    mrmd_batch* b = d->b;
    const int32_t N = b->N;
    const int64_t S = d->dc.steps, C = d->dc.checkpointInterval, W = d->dc.window;
    const double dt = b->cfg.dt, h = 0.5 * dt;  // unit masses
    const double c1 = b->B.ouDamping;
    // dL/d(rho_b) per kernel value
    std::vector<double> coef(d->hRho.size());
    const double scale = 1.0 / ((double)W * d->area);
    const double uniform = (double)N / (d->Lx * d->area);
    for (size_t k = 0; k < coef.size(); ++k) coef[k] = 2.0 * (d->hRho[k] * scale - uniform) * scale;
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    int rc = h2d(ctx, d->coef, coef.data(), sizeof(double) * coef.size());
    for (void* p : {(void*)d->xbar, (void*)d->vbar, (void*)d->Fbar})
        if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMemsetAsync(p, 0, sizeof(double4) * (size_t)N, ctx->stream), "adj");
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMemsetAsync(d->grad, 0, 2 * sizeof(double), ctx->stream), "adj");
    if (rc == MRMD_OK)
        rc = check_cuda(ctx, cudaMemsetAsync(d->tfGrad, 0, sizeof(double) * (size_t)std::max(d->nBins, 1), ctx->stream),
                        "adj");
    const unsigned g = grid_for(ctx, N, TB);
    AdjArgs A{};
    A.a = d->adj;
    A.af = d->adjf;
    A.xbar = d->xbar;
    A.grad = d->grad;
    A.tfGrad = d->tfGrad;
    A.L = make_ljdiff(d->eps, d->sig, d->rc, d->rcap, d->shifted);
    A.Lf = to_float(A.L);
    const bool mixed = b->cfg.precision == MRMD_PREC_MIXED;
    const int64_t segs = (S + C - 1) / C;
    for (int64_t sg = segs - 1; sg >= 0 && rc == MRMD_OK; --sg)
    {
        // recompute the segment from its checkpoint, keeping the pre-force positions
        const int64_t st0 = sg * C, st1 = std::min(S, st0 + C);
        rc = snapshot(ctx, b, d->ckpt[(size_t)sg], false);
        b->steps = st0;
        b->needRebuild = true;
        if (rc == MRMD_OK) rc = refresh_step_flags(ctx, b);
        for (int64_t st = st0; st < st1 && rc == MRMD_OK; ++st)
        {
            rc = step(ctx, b, st, true);
            if (rc == MRMD_OK)
                rc = check_cuda(ctx, cudaMemcpyAsync(d->x2 + (st - st0) * N, b->B.pos, sizeof(double4) * (size_t)N,
                                                     cudaMemcpyDeviceToDevice, ctx->stream),
                                "x2");
        }
        // adjoint steps, last to first.  Each step uses the forward's own pair
        // set: ghosts and list rebuilt from the positions of the forward's
        // rebuild step, ghost positions then moved with their sources.
        const int64_t K = b->cfg.tuning.rebuildInterval;
        int64_t builtFor = -1;
        for (int64_t st = st1 - 1; st >= st0 && rc == MRMD_OK; --st)
        {
            const int64_t rb = st - st % K;
            if (rb != builtFor)
            {
                rc = check_cuda(ctx, cudaMemcpyAsync(b->B.pos, d->x2 + (rb - st0) * N, sizeof(double4) * (size_t)N,
                                                     cudaMemcpyDeviceToDevice, ctx->stream),
                                "x2");
                if (rc == MRMD_OK) rc = rebuild_checked(ctx, b, false);
                builtFor = rb;
            }
            if (rc == MRMD_OK)
                rc = check_cuda(ctx, cudaMemcpyAsync(b->B.pos, d->x2 + (st - st0) * N, sizeof(double4) * (size_t)N,
                                                     cudaMemcpyDeviceToDevice, ctx->stream),
                                "x2");
            if (rc == MRMD_OK) rc = derive_locals(ctx, b);
            if (rc == MRMD_OK) rc = update_ghosts(ctx, b);
            if (rc != MRMD_OK) break;
            k_adj_prepare<<<g, TB, 0, ctx->stream>>>(d->Fbar, d->vbar, d->adj, N, h);
            rc = after_launch(ctx, "adj prepare");
            if (rc == MRMD_OK && mixed)
            {
                k_adj_float<<<g, TB, 0, ctx->stream>>>(d->adj, b->B.lam, N, d->adjf);
                rc = after_launch(ctx, "adj float");
            }
            if (rc == MRMD_OK)
            {
                const unsigned ga = (unsigned)div_up((int64_t)N * ADJ_TPR, TB);
                if (mixed)
                    k_adj_force<true, ADJ_TPR><<<ga, TB, 0, ctx->stream>>>(b->B, A);
                else
                    k_adj_force<false, ADJ_TPR><<<ga, TB, 0, ctx->stream>>>(b->B, A);
                rc = after_launch(ctx, "adj force");
            }
            if (rc == MRMD_OK && st >= S - W)
            {
                k_loss_grad<<<g, TB, 0, ctx->stream>>>(b->B, loss_dev(d), d->xbar);
                rc = after_launch(ctx, "loss grad");
            }
            if (rc == MRMD_OK)
            {
                k_adj_vv<<<g, TB, 0, ctx->stream>>>(d->xbar, d->vbar, d->Fbar, N, 0.5 * dt, c1, h);
                rc = after_launch(ctx, "adj vv");
            }
        }
    }
    double gr[2] = {0.0, 0.0};
    if (rc == MRMD_OK) rc = d2h(ctx, gr, d->grad, sizeof(gr));
    if (rc == MRMD_OK && gradTable && d->nBins) rc = d2h(ctx, gradTable, d->tfGrad, sizeof(double) * (size_t)d->nBins);
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    if (gradEpsilon) *gradEpsilon = gr[0];
    if (gradSigma) *gradSigma = gr[1];
    return MRMD_OK;
}

int mrmd_diff_force_vjp(mrmd_ctx* ctx, mrmd_diff* d, const double* tfTable, double epsilon, double sigma,
                        const double* adjoint3, double* force3, double* xbar3, double* gradTable, double* gradEpsilon,
                        double* gradSigma)
{
    if (!ctx || !d || !adjoint3 || !(epsilon > 0.0) || !(sigma > 0.0)) return MRMD_ERR_ARG;
    mrmd_batch* b = d->b;
    const size_t N = (size_t)b->N;
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    int rc = restore_initial(ctx, d);
    if (rc == MRMD_OK) rc = set_params(ctx, d, tfTable, epsilon, sigma);
    if (rc == MRMD_OK) rc = eval_forces(ctx, b);
    std::vector<double4> h(N);
    if (rc == MRMD_OK && force3) rc = d2h(ctx, h.data(), b->B.force, sizeof(double4) * N);
    if (rc == MRMD_OK && force3)
        for (size_t i = 0; i < N; ++i)
        {
            force3[3 * i] = h[i].x;
            force3[3 * i + 1] = h[i].y;
            force3[3 * i + 2] = h[i].z;
        }
    for (size_t i = 0; i < N; ++i) h[i] = make_double4(adjoint3[3 * i], adjoint3[3 * i + 1], adjoint3[3 * i + 2], 0.0);
    if (rc == MRMD_OK) rc = h2d(ctx, d->adj, h.data(), sizeof(double4) * N);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMemsetAsync(d->xbar, 0, sizeof(double4) * N, ctx->stream), "vjp");
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMemsetAsync(d->grad, 0, 2 * sizeof(double), ctx->stream), "vjp");
    if (rc == MRMD_OK)
        rc = check_cuda(ctx, cudaMemsetAsync(d->tfGrad, 0, sizeof(double) * (size_t)std::max(d->nBins, 1), ctx->stream),
                        "vjp");
    if (rc == MRMD_OK)
    {
        AdjArgs A{};
        A.a = d->adj;
        A.af = d->adjf;
        A.xbar = d->xbar;
        A.grad = d->grad;
        A.tfGrad = d->tfGrad;
        A.L = make_ljdiff(epsilon, sigma, d->rc, d->rcap, d->shifted);
        A.Lf = to_float(A.L);
        if (b->cfg.precision == MRMD_PREC_MIXED)
        {
            k_adj_float<<<grid_for(ctx, (int64_t)N, TB), TB, 0, ctx->stream>>>(d->adj, b->B.lam, (int32_t)N, d->adjf);
            k_adj_force<true, ADJ_TPR><<<(unsigned)div_up((int64_t)N * ADJ_TPR, TB), TB, 0, ctx->stream>>>(b->B, A);
        }
        else
            k_adj_force<false, ADJ_TPR><<<(unsigned)div_up((int64_t)N * ADJ_TPR, TB), TB, 0, ctx->stream>>>(b->B, A);
        rc = after_launch(ctx, "adj force");
    }
    if (rc == MRMD_OK && xbar3) rc = d2h(ctx, h.data(), d->xbar, sizeof(double4) * N);
    if (rc == MRMD_OK && xbar3)
        for (size_t i = 0; i < N; ++i)
        {
            xbar3[3 * i] = h[i].x;
            xbar3[3 * i + 1] = h[i].y;
            xbar3[3 * i + 2] = h[i].z;
        }
    double gr[2] = {0.0, 0.0};
    if (rc == MRMD_OK) rc = d2h(ctx, gr, d->grad, sizeof(gr));
    if (rc == MRMD_OK && gradTable && d->nBins) rc = d2h(ctx, gradTable, d->tfGrad, sizeof(double) * (size_t)d->nBins);
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    if (gradEpsilon) *gradEpsilon = gr[0];
    if (gradSigma) *gradSigma = gr[1];
    d->haveForward = false;
    return MRMD_OK;
}

int mrmd_diff_get_state(mrmd_ctx* ctx, mrmd_diff* d, double* pos3, double* vel3)
{
    if (!ctx || !d) return MRMD_ERR_ARG;
    return mrmd_batch_get_state(ctx, d->b, pos3, vel3, nullptr);
}

}  // extern "C"
