// AdResS: weighting_function::Slab + UpdateMolecules, ContributeMoleculeForceToAtoms
// and action::LJ_IdealGas (weighted molecule-pair LJ, drift force and the
// drift-compensation energy histogram).
#include <cmath>
#include <vector>

#include "common.cuh"
#include "lj_impl.cuh"
#include "lj_mixed.cuh"
#include "nlist_impl.cuh"
#include "adress_impl.cuh"

using namespace mrmd_impl;

namespace
{
constexpr int TB = 256;
__global__ void k_update_molecules(mrmd_molecules m, const double4* __restrict__ apos,
                                   const double* __restrict__ relMass, int64_t n, SlabDev s)
{
    // action/UpdateMolecules.hpp:39-69
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t a0 = m.atomsOffset[i], a1 = a0 + m.numAtoms[i];
        double x = 0.0, y = 0.0, z = 0.0;
        for (int64_t a = a0; a < a1; ++a)
        {
            const double4 p = apos[a];
            const double w = relMass[a];
            x = __dadd_rn(x, __dmul_rn(p.x, w));
            y = __dadd_rn(y, __dmul_rn(p.y, w));
            z = __dadd_rn(z, __dmul_rn(p.z, w));
        }
        reinterpret_cast<double4*>(m.pos)[i] = make_double4(x, y, z, 0.0);
        double lam, mod, gx;
        slab_eval(s, x, lam, mod, gx);
        m.lambda[i] = lam;
        m.modulatedLambda[i] = mod;
        reinterpret_cast<double4*>(m.gradLambda)[i] = make_double4(gx, 0.0, 0.0, 0.0);
    }
}

__global__ void k_contribute(mrmd_molecules m, double4* __restrict__ aforce, const double* __restrict__ relMass,
                             int64_t n)
{
    // action/ContributeMoleculeForceToAtoms.cpp:32-47
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double4 fm = reinterpret_cast<const double4*>(m.force)[i];
        const int64_t a0 = m.atomsOffset[i], a1 = a0 + m.numAtoms[i];
        for (int64_t a = a0; a < a1; ++a)
        {
            const double w = relMass[a];
            double4 f = aforce[a];
            f.x = __dadd_rn(f.x, __dmul_rn(w, fm.x));
            f.y = __dadd_rn(f.y, __dmul_rn(w, fm.y));
            f.z = __dadd_rn(f.z, __dmul_rn(w, fm.z));
            aforce[a] = f;
        }
    }
}

struct LJIGArgs
{
    const double4* apos;
    double* aforce;
    const int32_t* atype;
    const float4* hi;  // mixed form split coordinates (else null)
    const float4* lo;
    mrmd_molecules m;
    const int32_t* counts;
    const int32_t* nbrs;
    int64_t cap;
    int64_t nMol;      // list rows
    int64_t begin;     // molecule of list row 0
    const LJDev* table;
    int32_t numTypes;
    double rcSqr;
    RcSq rc2;
    int32_t sampling;
    double* compEnergy;   // [200][numTypes]
    double* compCounter;  // [200][numTypes]
    const double* meanComp;
    double* energyOut;
};

template <bool MIXED>
__global__ void __launch_bounds__(128) k_ljig(LJIGArgs A)
{
    // action/LJ_IdealGas.cpp:52-225, one thread per local molecule alpha
    __shared__ double red[64];
    double sumEnergy = 0.0, dummy = 0.0;
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row < A.nMol)
    {
        const int64_t alpha = A.begin + row;
        double fA[3] = {0.0, 0.0, 0.0};
        const double modA = A.m.modulatedLambda[alpha];
        int binAlpha = -1;
        if (is_hy(modA)) binAlpha = comp_bin(A.m.lambda[alpha]);
        const double4 gA = reinterpret_cast<const double4*>(A.m.gradLambda)[alpha];
        const int64_t sA = A.m.atomsOffset[alpha], eA = sA + A.m.numAtoms[alpha];
        const int32_t cnt = A.counts[row];
        for (int32_t k = 0; k < cnt; ++k)
        {
            const int64_t beta = A.nbrs[mrmd_dev::nbr_row(row, A.cap) + 32 * (int64_t)k];
            double fB[3] = {0.0, 0.0, 0.0};
            const double modB = A.m.modulatedLambda[beta];
            if (is_cg(modA) && is_cg(modB)) continue;
            const double4 gB = reinterpret_cast<const double4*>(A.m.gradLambda)[beta];
            const double weighting = 0.5 * (modA + modB);
            const bool hyPair = is_hy(modA) || is_hy(modB);
            const int64_t sB = A.m.atomsOffset[beta], eB = sB + A.m.numAtoms[beta];
            int binBeta = -1;
            if (A.sampling && is_hy(modB)) binBeta = comp_bin(A.m.lambda[beta]);
            for (int64_t idx = sA; idx < eA; ++idx)
            {
                const double4 pi = A.apos[idx];
                double fi[3] = {0.0, 0.0, 0.0};
                const int32_t ti = A.atype[idx];
                for (int64_t jdx = sB; jdx < eB; ++jdx)
                {
                    const int32_t tj = A.atype[jdx];
                    const LJDev& p = A.table[ti * A.numTypes + tj];
                    double ff, e, dx, dy, dz;
                    if (MIXED)
                    {
                        PairMixed q;
                        if (!pair_mixed(A.hi[idx], A.lo[idx], A.hi[jdx], A.lo[jdx], p, A.rc2, q)) continue;
                        ff = (double)q.ff.h + (double)q.ff.l;
                        e = q.e;
                        dx = (double)q.dh.x + (double)q.dl.x;
                        dy = (double)q.dh.y + (double)q.dl.y;
                        dz = (double)q.dh.z + (double)q.dl.z;
                    }
                    else
                    {
                        const double4 pj = A.apos[jdx];
                        dx = pi.x - pj.x;
                        dy = pi.y - pj.y;
                        dz = pi.z - pj.z;
                        const double distSqr = dx * dx + dy * dy + dz * dz;
                        if (distSqr > A.rcSqr) continue;
                        lj_eval_fp64(p, distSqr, ff, e);
                    }
                    const double ffactor = ff * weighting;
                    fi[0] += dx * ffactor;
                    fi[1] += dy * ffactor;
                    fi[2] += dz * ffactor;
                    atomicAdd(A.aforce + 4 * jdx + 0, -(dx * ffactor));
                    atomicAdd(A.aforce + 4 * jdx + 1, -(dy * ffactor));
                    atomicAdd(A.aforce + 4 * jdx + 2, -(dz * ffactor));
                    sumEnergy += e * weighting;
                    const double Vij = 0.5 * e;
                    if (hyPair)
                    {
                        fA[0] += -Vij * gA.x;
                        fA[1] += -Vij * gA.y;
                        fA[2] += -Vij * gA.z;
                        fB[0] += -Vij * gB.x;
                        fB[1] += -Vij * gB.y;
                        fB[2] += -Vij * gB.z;
                        if (A.sampling)
                        {
                            if (is_hy(modA) && binAlpha != -1)
                                atomicAdd(A.compEnergy + binAlpha * A.numTypes + ti, Vij);
                            if (is_hy(modB) && binBeta != -1)
                                atomicAdd(A.compEnergy + binBeta * A.numTypes + tj, Vij);
                        }
                    }
                }
                atomicAdd(A.aforce + 4 * idx + 0, fi[0]);
                atomicAdd(A.aforce + 4 * idx + 1, fi[1]);
                atomicAdd(A.aforce + 4 * idx + 2, fi[2]);
            }
            double* mf = A.m.force + 4 * beta;
            atomicAdd(mf + 0, fB[0]);
            atomicAdd(mf + 1, fB[1]);
            atomicAdd(mf + 2, fB[2]);
        }
        if (A.sampling && is_hy(modA) && binAlpha != -1)
            for (int64_t a = sA; a < eA; ++a) atomicAdd(A.compCounter + binAlpha * A.numTypes + A.atype[a], 1.0);
        if (is_hy(modA) && binAlpha != -1)
        {
            const double me = A.meanComp[binAlpha * A.numTypes + A.atype[sA]];
            fA[0] += me * gA.x;
            fA[1] += me * gA.y;
            fA[2] += me * gA.z;
        }
        double* mf = A.m.force + 4 * alpha;
        atomicAdd(mf + 0, fA[0]);
        atomicAdd(mf + 1, fA[1]);
        atomicAdd(mf + 2, fA[2]);
    }
    mrmd_dev::block_sum2(sumEnergy, dummy, red);
    if (threadIdx.x == 0) atomicAdd(A.energyOut, sumEnergy);
}

__global__ void k_update_mean_comp(double* __restrict__ energy, double* __restrict__ counter,
                                   double* __restrict__ mean, int64_t n, double factor)
{
    // action/LJ_IdealGas.cpp:21-50
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    {
        if (counter[k] < 0.5) continue;
        const double e = energy[k] / counter[k];
        mean[k] = (factor * mean[k] + e) / (factor + 1.0);
        energy[k] = 0.0;
        counter[k] = 0.0;
    }
}

}  // namespace

struct mrmd_ljig
{
    int64_t numTypes = 1;
    double rcSqr = 0.0;
    std::vector<mrmd_lj_params> table;
    LJDev* dTable = nullptr;
    double* comp = nullptr;  // [3][200][numTypes]: energy, counter, mean
    int64_t runCounter = 0;
    int64_t samplingInterval = 200;
    int64_t updateInterval = 20000;
};

extern "C" {

int mrmd_update_molecules(mrmd_ctx* ctx, mrmd_molecules* m, const mrmd_atoms* a, const mrmd_slab* slab)
{
    if (!ctx || !m || !a || !slab) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(slab->hybridRegionDiameter > 0.0 || slab->interfaceType == 1, ctx, "hybrid width must be > 0");
    const int64_t n = m->numLocal + m->numGhost;
    if (n == 0) return MRMD_OK;
    k_update_molecules<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(*m, reinterpret_cast<const double4*>(a->pos),
                                                                      a->relativeMass, n, to_slab(slab));
    MRMD_TRY(after_launch(ctx, "update_molecules"));
    return finish(ctx, "update_molecules");
}

int mrmd_contribute_molecule_force(mrmd_ctx* ctx, const mrmd_molecules* m, mrmd_atoms* a)
{
    if (!ctx || !m || !a) return MRMD_ERR_ARG;
    const int64_t n = m->numLocal + m->numGhost;
    if (n == 0) return MRMD_OK;
    k_contribute<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(*m, reinterpret_cast<double4*>(a->force),
                                                                a->relativeMass, n);
    MRMD_TRY(after_launch(ctx, "contribute_molecule_force"));
    return finish(ctx, "contribute_molecule_force");
}

int mrmd_ljig_create(mrmd_ctx* ctx, mrmd_ljig** out, int64_t numTypes, const double* cappingDistance,
                     const double* rc, const double* sigma, const double* epsilon, int doShift)
{
    if (!ctx || !out || !cappingDistance || !rc || !sigma || !epsilon) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(numTypes >= 1 && numTypes <= 64, ctx, "numTypes out of range");
    *out = nullptr;
    mrmd_ljig* s = new mrmd_ljig();
    s->numTypes = numTypes;
    const int64_t n2 = numTypes * numTypes;
    s->table.resize((size_t)n2);
    lj_table_host(s->table.data(), numTypes, cappingDistance, rc, sigma, epsilon, doShift);
    double rcMax = rc[0];
    for (int64_t t = 1; t < n2; ++t) rcMax = std::fmax(rcMax, rc[t]);
    s->rcSqr = rcMax * rcMax;  // LJ_IdealGas.cpp:290-291
    std::vector<LJDev> dev((size_t)n2);
    for (int64_t t = 0; t < n2; ++t) dev[(size_t)t] = to_dev(s->table[(size_t)t]);
    int rc2 = dmalloc(ctx, reinterpret_cast<void**>(&s->dTable), sizeof(LJDev) * (size_t)n2);
    if (rc2 == MRMD_OK)
        rc2 = h2d(ctx, s->dTable, dev.data(), sizeof(LJDev) * (size_t)n2);
    const size_t compBytes = sizeof(double) * 3 * COMP_BINS * (size_t)numTypes;
    if (rc2 == MRMD_OK) rc2 = dmalloc(ctx, reinterpret_cast<void**>(&s->comp), compBytes);
    if (rc2 == MRMD_OK) rc2 = dzero(ctx, s->comp, compBytes);
    if (rc2 != MRMD_OK)
    {
        dfree(s->dTable);
        dfree(s->comp);
        delete s;
        return rc2;
    }
    *out = s;
    return MRMD_OK;
}

int mrmd_ljig_destroy(mrmd_ctx* ctx, mrmd_ljig* s)
{
    if (!s) return MRMD_OK;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(s->dTable);
    dfree(s->comp);
    delete s;
    return MRMD_OK;
}

int mrmd_ljig_set_intervals(mrmd_ljig* s, int64_t samplingInterval, int64_t updateInterval)
{
    if (!s || samplingInterval < 1 || updateInterval < 1) return MRMD_ERR_ARG;
    s->samplingInterval = samplingInterval;
    s->updateInterval = updateInterval;
    return MRMD_OK;
}

}  // extern "C"

namespace mrmd_impl
{
// LJ_IdealGas::run (LJ_IdealGas.cpp:227-260) without any host read-back:
// the energy is added to *ev (device, zeroed by the caller).  For the mixed
// form `hi`/`lo` may hold split coordinates already computed for the list's
// grid (else they are computed into context scratch).
int ljig_run_async(mrmd_ctx* ctx, mrmd_ljig* s, mrmd_molecules* m, const mrmd_nlist* nl, mrmd_atoms* a,
                   int precision, double* ev, const float4* hiIn, const float4* loIn)
{
    const int sampling = (s->runCounter % s->samplingInterval) == 0;
    const int64_t nb = COMP_BINS * s->numTypes;
    LJIGArgs A{};
    A.apos = reinterpret_cast<const double4*>(a->pos);
    A.aforce = a->force;
    A.atype = a->type;
    A.m = *m;
    A.counts = nl->counts;
    A.nbrs = nl->nbrs;
    A.cap = nl->maxNeighbors;
    A.nMol = nl->rows;
    A.begin = nl->begin;
    A.table = s->dTable;
    A.numTypes = (int32_t)s->numTypes;
    A.rcSqr = s->rcSqr;
    A.rc2 = make_rcsq(s->rcSqr);
    A.sampling = sampling;
    A.compEnergy = s->comp;
    A.compCounter = s->comp + nb;
    A.meanComp = s->comp + 2 * nb;
    A.energyOut = ev;
    if (A.nMol > 0)
    {
        const unsigned grid = (unsigned)div_up(A.nMol, 128);
        if (precision == MRMD_PREC_MIXED)
        {
            if (hiIn && loIn)
            {
                A.hi = hiIn;
                A.lo = loIn;
            }
            else
            {
                const int64_t nAll = a->numLocal + a->numGhost;
                float4* hi = static_cast<float4*>(scratch(ctx, sizeof(float4) * 2 * (size_t)nAll));
                if (!hi) return MRMD_ERR_OOM;
                MRMD_TRY(split_coords(ctx, a->pos, nAll, split_params_for(nl), hi, hi + nAll));
                A.hi = hi;
                A.lo = hi + nAll;
            }
            k_ljig<true><<<grid, 128, 0, ctx->stream>>>(A);
        }
        else
        {
            k_ljig<false><<<grid, 128, 0, ctx->stream>>>(A);
        }
        MRMD_TRY(after_launch(ctx, "ljig"));
    }
    if (s->runCounter % s->updateInterval == 0)
    {
        k_update_mean_comp<<<grid_for(ctx, nb, TB), TB, 0, ctx->stream>>>(s->comp, s->comp + nb, s->comp + 2 * nb,
                                                                          nb, 10.0);
        MRMD_TRY(after_launch(ctx, "update_mean_comp"));
    }
    ++s->runCounter;
    return MRMD_OK;
}
}  // namespace mrmd_impl

extern "C" {

int mrmd_ljig_run(mrmd_ctx* ctx, mrmd_ljig* s, mrmd_molecules* m, const mrmd_nlist* nl, mrmd_atoms* a,
                  int precision, double* energy)
{
    // action/LJ_IdealGas.cpp:227-260
    if (!ctx || !s || !m || !nl || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(precision == MRMD_PREC_FP64 || precision == MRMD_PREC_MIXED, ctx, "bad precision");
    MRMD_TRY(check_list_fits(ctx, nl, m->numLocal, m->numLocal + m->numGhost));
    double* ev = ctx->devScalars + 32;
    MRMD_CUDA(ctx, cudaMemsetAsync(ev, 0, sizeof(double), ctx->stream));
    MRMD_TRY(ljig_run_async(ctx, s, m, nl, a, precision, ev, nullptr, nullptr));
    MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 32, ev, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (energy) *energy = ctx->hostScalars[32];
    return MRMD_OK;
}

int mrmd_ljig_get_compensation(mrmd_ctx* ctx, const mrmd_ljig* s, double* mean, double* energy, double* counter,
                               int64_t* runCounter)
{
    if (!ctx || !s) return MRMD_ERR_ARG;
    const size_t nb = COMP_BINS * (size_t)s->numTypes;
    if (energy) MRMD_TRY(d2h(ctx, energy, s->comp, sizeof(double) * nb));
    if (counter) MRMD_TRY(d2h(ctx, counter, s->comp + nb, sizeof(double) * nb));
    if (mean) MRMD_TRY(d2h(ctx, mean, s->comp + 2 * nb, sizeof(double) * nb));
    if (runCounter) *runCounter = s->runCounter;
    return MRMD_OK;
}

int mrmd_ljig_set_compensation(mrmd_ctx* ctx, mrmd_ljig* s, const double* mean)
{
    if (!ctx || !s || !mean) return MRMD_ERR_ARG;
    const size_t nb = COMP_BINS * (size_t)s->numTypes;
    MRMD_TRY(h2d(ctx, s->comp + 2 * nb, mean, sizeof(double) * nb));
    return MRMD_OK;
}

}  // extern "C"
