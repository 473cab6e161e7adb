// impl::CoulombDSF: damped shifted force Coulomb (Fennell & Gezelter,
// DOI 10.1140/epjst/e2016-60151-6, eqs 15-16) as a device pair function, and
// a half-list pair force that applies it with the atoms' charges.
//
// The reference ships the pair function alone (action/CoulombDSF.hpp:39-83;
// nothing calls it).  The pair force here follows LennardJones::apply's loop
// (action/LennardJones.hpp:135-206) on the same neighbour list: one thread
// per local atom, i-force in registers, j-force scattered with FP64 atomics,
// energy and virial reduced per block.  FP64 throughout: the pair function
// needs exp() and a division per pair, and the shifts are differences of
// nearly equal terms near the cutoff.
#include <cmath>

#include "common.cuh"
#include "nlist_impl.cuh"

using namespace mrmd_impl;

namespace
{
constexpr int TBC = 128;
constexpr double INV_SQRTPI = 0.56418958354775628695;  // 1 / sqrt(pi)
constexpr double PREFACTOR = 138.935458;               // CoulombDSF.hpp:57

// util::approxErfc (util/math.hpp:57-70): Abramowitz & Stegun 7.1.26,
// erfc(x) ~ t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-x^2), t = 1/(1 + p x).
__host__ __device__ __forceinline__ double approx_erfc(double x, double& expX2)
{
    const double p = 0.3275911;
    const double a1 = 0.254829592;
    const double a2 = -0.284496736;
    const double a3 = 1.421413741;
    const double a4 = -1.453152027;
    const double a5 = 1.061405429;
    const double t = 1.0 / (1.0 + p * x);
    expX2 = exp(-x * x);
    return t * (a1 + t * (a2 + t * (a3 + t * (a4 + t * a5)))) * expX2;
}

// computeForce (CoulombDSF.hpp:52-62, returned divided by r^2) and
// computeEnergy (:64-74); both share r and the erfc evaluation.
__device__ __forceinline__ void dsf_eval(const mrmd_coulomb_dsf_params& c, double distSqr, double q1, double q2,
                                         double& ff, double& e)
{
    const double r = sqrt(distSqr);
    const double prefac = PREFACTOR * q1 * q2;
    double expX2;
    const double erfc = approx_erfc(c.alpha * r, expX2);
    ff = prefac * (erfc / r + 2.0 * c.alpha * INV_SQRTPI * expX2 + r * c.forceShift) / distSqr;
    e = prefac * (erfc / r - c.energyShift - c.forceShift * (r - c.rc));
}

__global__ void k_dsf_eval(const mrmd_coulomb_dsf_params c, int64_t n, const double* __restrict__ distSqr,
                           const double* __restrict__ q1, const double* __restrict__ q2, double* __restrict__ ff,
                           double* __restrict__ e)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dsf_eval(c, distSqr[i], q1[i], q2[i], ff[i], e[i]);
}

__global__ void __launch_bounds__(TBC) k_dsf_apply(const double4* __restrict__ pos, double* __restrict__ force,
                                                  const double* __restrict__ charge, const mrmd_coulomb_dsf_params c,
                                                  const int32_t* __restrict__ counts,
                                                  const int32_t* __restrict__ nbrs, int64_t cap, int64_t n,
                                                  int64_t begin, double* __restrict__ ev)
{
    __shared__ double red[64];
    double energy = 0.0, virial = 0.0;
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row < n)
    {
        const int64_t i = begin + row;  // list row `row` belongs to particle begin + row
        const double4 pi = pos[i];
        const double qi = charge[i];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        const int32_t cnt = counts[row];
        const int32_t* __restrict__ col = nbrs + mrmd_dev::nbr_row(row, cap);
        for (int32_t k = 0; k < cnt; ++k)
        {
            const int32_t j = __ldg(col + 32 * (int64_t)k);
            const double4 pj = mrmd_dev::ldg4(pos + j);
            const double dx = pi.x - pj.x;
            const double dy = pi.y - pj.y;
            const double dz = pi.z - pj.z;
            const double distSqr = dx * dx + dy * dy + dz * dz;
            if (distSqr > c.rcSqr) continue;
            double ff, e;
            dsf_eval(c, distSqr, qi, __ldg(charge + j), ff, e);
            energy += e;
            virial -= 0.5 * ff * distSqr;
            const double gx = dx * ff, gy = dy * ff, gz = dz * ff;
            fx += gx;
            fy += gy;
            fz += gz;
            atomicAdd(force + 4 * (int64_t)j + 0, -gx);
            atomicAdd(force + 4 * (int64_t)j + 1, -gy);
            atomicAdd(force + 4 * (int64_t)j + 2, -gz);
        }
        atomicAdd(force + 4 * i + 0, fx);
        atomicAdd(force + 4 * i + 1, fy);
        atomicAdd(force + 4 * i + 2, fz);
    }
    mrmd_dev::block_sum2(energy, virial, red);
    if (threadIdx.x == 0)
    {
        atomicAdd(ev + 0, energy);
        atomicAdd(ev + 1, virial);
    }
}
}  // namespace

extern "C" {

int mrmd_coulomb_dsf_init(mrmd_coulomb_dsf_params* out, double rc, double alpha)
{
    // CoulombDSF.hpp:76-83: the shifts use the exact erfc
    if (!out || !(rc > 0.0) || !(alpha > 0.0)) return MRMD_ERR_ARG;
    out->alpha = alpha;
    out->rc = rc;
    out->rcSqr = rc * rc;
    const double erfc = std::erfc(alpha * rc);
    const double ex = std::exp(-alpha * alpha * out->rcSqr);
    out->forceShift = -(erfc / out->rcSqr + 2.0 * INV_SQRTPI * alpha * ex / rc);
    out->energyShift = erfc / rc;
    return MRMD_OK;
}

int mrmd_coulomb_dsf_eval(mrmd_ctx* ctx, const mrmd_coulomb_dsf_params* c, int64_t n, const double* distSqr,
                          const double* q1, const double* q2, double* force, double* energy)
{
    if (!ctx || !c || n < 0 || (n > 0 && (!distSqr || !q1 || !q2 || !force || !energy))) return MRMD_ERR_ARG;
    if (n == 0) return MRMD_OK;
    double* d = static_cast<double*>(scratch(ctx, sizeof(double) * 5 * (size_t)n));
    if (!d) return MRMD_ERR_OOM;
    MRMD_CUDA(ctx, cudaMemcpyAsync(d, distSqr, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    MRMD_CUDA(ctx, cudaMemcpyAsync(d + n, q1, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    MRMD_CUDA(ctx, cudaMemcpyAsync(d + 2 * n, q2, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    k_dsf_eval<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(*c, n, d, d + n, d + 2 * n, d + 3 * n, d + 4 * n);
    MRMD_TRY(after_launch(ctx, "coulomb_dsf_eval"));
    MRMD_CUDA(ctx, cudaMemcpyAsync(force, d + 3 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaMemcpyAsync(energy, d + 4 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "coulomb_dsf_eval");
}

int mrmd_coulomb_dsf_apply(mrmd_ctx* ctx, const mrmd_coulomb_dsf_params* c, mrmd_atoms* a, const mrmd_nlist* nl,
                           double* energy, double* virial)
{
    if (!ctx || !c || !a || !nl) return MRMD_ERR_ARG;
    MRMD_TRY(check_list_fits(ctx, nl, a->numLocal, a->numLocal + a->numGhost));
    double* ev = ctx->devScalars + 12;
    MRMD_CUDA(ctx, cudaMemsetAsync(ev, 0, 2 * sizeof(double), ctx->stream));
    const int64_t n = nl->rows;
    if (n > 0)
    {
        k_dsf_apply<<<(unsigned)div_up(n, TBC), TBC, 0, ctx->stream>>>(
            reinterpret_cast<const double4*>(a->pos), a->force, a->charge, *c, nl->counts, nl->nbrs,
            nl->maxNeighbors, n, nl->begin, ev);
        MRMD_TRY(after_launch(ctx, "coulomb_dsf"));
    }
    if (energy || virial)
    {
        MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 12, ev, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (energy) *energy = ctx->hostScalars[12];
        if (virial) *virial = ctx->hostScalars[13];
        return MRMD_OK;
    }
    return finish(ctx, "coulomb_dsf_apply");
}

}  // extern "C"
