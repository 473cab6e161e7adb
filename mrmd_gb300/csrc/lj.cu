// action::LennardJones: capped, optionally shifted LJ on a half Verlet list.
//
// FP64 form: one thread per local atom i (atoms are cell-sorted by the
// stepper, so a warp's neighbours share cache lines), i-force in registers,
// j-force scattered with FP64 atomics into the 32-byte atom sector, energy
// and virial reduced per block and added once per block.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "lj_impl.cuh"
#include "nlist_impl.cuh"

using namespace mrmd_impl;

namespace mrmd_impl
{
void lj_force_energy_host(const mrmd_lj_params* t, double distSqr, int64_t typeIdx, double* ff, double* e)
{
    // action/LennardJones.hpp:52-78 evaluated on the host with IEEE doubles
    const mrmd_lj_params& p = t[typeIdx];
    if (distSqr >= p.cappingDistanceSqr)
    {
        const double frac2 = 1.0 / distSqr;
        const double frac6 = frac2 * frac2 * frac2;
        *ff = frac6 * (p.ff1 * frac6 - p.ff2) * frac2;
        *e = frac6 * (p.ef1 * frac6 - p.ef2) - p.shift;
        return;
    }
    const double dist = std::sqrt(distSqr);
    *ff = p.cappingCoeff / dist;
    *e = p.energyAtCappingPoint - (dist - p.cappingDistance) * p.cappingCoeff - p.shift;
}

void lj_table_host(mrmd_lj_params* out, int64_t numTypes, const double* cap, const double* rc,
                   const double* sigma, const double* epsilon, int isShifted)
{
    // constructor action/LennardJones.cpp:81-116, precompute :61-79
    for (int64_t t = 0; t < numTypes * numTypes; ++t)
    {
        const double sig2 = sigma[t] * sigma[t];
        const double sig6 = sig2 * sig2 * sig2;
        std::memset(&out[t], 0, sizeof(mrmd_lj_params));
        out[t].ff1 = 48.0 * epsilon[t] * sig6 * sig6;
        out[t].ff2 = 24.0 * epsilon[t] * sig6;
        out[t].ef1 = 4.0 * epsilon[t] * sig6 * sig6;
        out[t].ef2 = 4.0 * epsilon[t] * sig6;
        out[t].rcSqr = rc[t] * rc[t];
        out[t].cappingDistance = cap[t];
    }
    for (int64_t t = 0; t < numTypes * numTypes; ++t)
    {
        const double capDist = out[t].cappingDistance;
        out[t].cappingDistance = 0.0;
        out[t].cappingDistanceSqr = 0.0;
        double ff, e;
        lj_force_energy_host(out, capDist * capDist, t, &ff, &e);
        out[t].cappingCoeff = ff * capDist;
        out[t].energyAtCappingPoint = e;
        out[t].cappingDistance = capDist;
        out[t].cappingDistanceSqr = capDist * capDist;
        if (isShifted)
        {
            lj_force_energy_host(out, out[t].rcSqr, t, &ff, &e);
            out[t].shift = e;
        }
    }
}

namespace
{
constexpr int LJ_TB = 128;

template <bool PRED, bool MULTI>
__global__ void __launch_bounds__(LJ_TB) k_lj_fp64(
    const double4* __restrict__ pos, double* __restrict__ force, const int32_t* __restrict__ type,
    const LJDev p0, const LJDev* __restrict__ table, int32_t numTypesIndex, double rcSqr,
    const int32_t* __restrict__ counts, const int32_t* __restrict__ nbrs, int64_t cap, int64_t n,
    int64_t begin, int64_t nAll, mrmd_dev::Pred pred, double* __restrict__ ev)
{
    __shared__ double red[64];
    double energy = 0.0, virial = 0.0;
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row < n)
    {
        // list row `row` belongs to particle begin + row (the list's range)
        const int64_t i = begin + row;
        const double4 pi = pos[i];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        const int32_t cnt = counts[row];
        const int32_t ti = MULTI ? type[i] * numTypesIndex : 0;
        const int32_t* __restrict__ col = nbrs + mrmd_dev::nbr_row(row, cap);
        for (int32_t k = 0; k < cnt; ++k)
        {
            const int32_t j = __ldg(col + 32 * (int64_t)k);
            if (!MRMD_IN_BOUNDS(j, nAll)) continue;
            const double4 pj = mrmd_dev::ldg4(pos + j);
            if (PRED && !mrmd_dev::pred2(pred, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z)) continue;
            const double dx = pi.x - pj.x;
            const double dy = pi.y - pj.y;
            const double dz = pi.z - pj.z;
            const double distSqr = dx * dx + dy * dy + dz * dz;
            if (distSqr > rcSqr) continue;
            const LJDev& p = MULTI ? table[ti + type[j]] : p0;
            double ff, e;
            lj_eval_fp64(p, distSqr, ff, e);
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

int lj_apply_fp64(mrmd_ctx* ctx, const mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl,
                  const mrmd_pred* pred, double* ev)
{
    const int64_t n = nl->rows;
    if (n == 0) return MRMD_OK;
    const bool usePred = pred != nullptr && pred->kind != MRMD_PRED_ALWAYS;
    const bool multi = lj->numTypes > 1;
    const mrmd_dev::Pred dp = to_dev_pred(pred);
    const unsigned grid = (unsigned)div_up(n, LJ_TB);
    const double4* pos = reinterpret_cast<const double4*>(a->pos);
#define LJ_LAUNCH(P, M)                                                                                \
    k_lj_fp64<P, M><<<grid, LJ_TB, 0, ctx->stream>>>(pos, a->force, a->type, lj->p0, lj->dTable,         \
                                                     (int32_t)lj->numTypesIndex, lj->rcSqr, nl->counts, \
                                                     nl->nbrs, nl->maxNeighbors, n, nl->begin, a->numLocal + a->numGhost, dp, ev)
    if (usePred && multi) LJ_LAUNCH(true, true);
    else if (usePred) LJ_LAUNCH(true, false);
    else if (multi) LJ_LAUNCH(false, true);
    else LJ_LAUNCH(false, false);
#undef LJ_LAUNCH
    return after_launch(ctx, "lj_fp64");
}
}  // namespace mrmd_impl

extern "C" {

int mrmd_lj_create(mrmd_ctx* ctx, mrmd_lj** out, int64_t numTypes, int64_t numTypesIndex,
                   const double* cappingDistance, const double* rc, const double* sigma,
                   const double* epsilon, int isShifted)
{
    if (!ctx || !out || !cappingDistance || !rc || !sigma || !epsilon) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(numTypes >= 1 && numTypes <= 64, ctx, "numTypes out of range");
    MRMD_CHECK_ARG(numTypesIndex >= 0 && numTypesIndex <= numTypes, ctx, "bad numTypesIndex");
    *out = nullptr;
    mrmd_lj* lj = new mrmd_lj();
    lj->numTypes = numTypes;
    lj->numTypesIndex = numTypesIndex;
    const int64_t n2 = numTypes * numTypes;
    lj->table.resize((size_t)n2);
    lj_table_host(lj->table.data(), numTypes, cappingDistance, rc, sigma, epsilon, isShifted);
    double rcMax = rc[0];
    for (int64_t t = 1; t < n2; ++t) rcMax = std::fmax(rcMax, rc[t]);
    lj->rcSqr = rcMax * rcMax;  // action/LennardJones.cpp:54-55
    std::vector<LJDev> dev((size_t)n2);
    for (int64_t t = 0; t < n2; ++t) dev[(size_t)t] = to_dev(lj->table[(size_t)t]);
    lj->p0 = dev[0];
    int rc2 = dmalloc(ctx, reinterpret_cast<void**>(&lj->dTable), sizeof(LJDev) * (size_t)n2);
    if (rc2 == MRMD_OK)
        rc2 = h2d(ctx, lj->dTable, dev.data(), sizeof(LJDev) * (size_t)n2);
    if (rc2 != MRMD_OK)
    {
        dfree(lj->dTable);
        delete lj;
        return rc2;
    }
    *out = lj;
    return MRMD_OK;
}

int mrmd_lj_destroy(mrmd_ctx* ctx, mrmd_lj* lj)
{
    if (!lj) return MRMD_OK;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(lj->dTable);
    delete lj;
    return MRMD_OK;
}

int mrmd_lj_get_params(const mrmd_lj* lj, mrmd_lj_params* out, int64_t count)
{
    if (!lj || !out) return MRMD_ERR_ARG;
    const int64_t n = (int64_t)lj->table.size();
    for (int64_t t = 0; t < count && t < n; ++t) out[t] = lj->table[(size_t)t];
    return MRMD_OK;
}

int mrmd_lj_apply(mrmd_ctx* ctx, mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl, const mrmd_pred* pred,
                  int precision, double* energy, double* virial)
{
    if (!ctx || !lj || !a || !nl) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(pred_valid(pred), ctx, "bad predicate");
    MRMD_CHECK_ARG(precision == MRMD_PREC_FP64 || precision == MRMD_PREC_MIXED, ctx, "bad precision");
    MRMD_TRY(check_list_fits(ctx, nl, a->numLocal, a->numLocal + a->numGhost));
    double* ev = ctx->devScalars + 16;
    MRMD_CUDA(ctx, cudaMemsetAsync(ev, 0, 2 * sizeof(double), ctx->stream));
    if (precision == MRMD_PREC_FP64)
        MRMD_TRY(lj_apply_fp64(ctx, lj, a, nl, pred, ev));
    else
        MRMD_TRY(lj_apply_mixed(ctx, lj, a, nl, pred, ev));
    if (energy || virial)
    {
        MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 16, ev, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (energy) *energy = ctx->hostScalars[16];
        if (virial) *virial = ctx->hostScalars[17];
        return MRMD_OK;
    }
    return finish(ctx, "lj_apply");
}

}  // extern "C"
