// Mixed-precision Lennard-Jones pair force.
//
// Positions stay FP64 in the atoms; before the pair kernel each coordinate
// c = x - origin (origin = the list's cell-grid corner) is split into
//   hi = c rounded to a multiple of 2^-q, q = 24 - ceil(log2(extent)),
//   lo = float(c - hi),
// so every hi is an integer multiple of 2^-q below 2^24 * 2^-q: the FP32
// difference hi_i - hi_j is exact, and dx = (hi_i - hi_j) + (lo_i - lo_j)
// carries ~2^-40 absolute accuracy.  r^2, 1/r^2, the force factor and the
// force products are evaluated in double-float (pairs of FP32), because the
// LJ force factor amplifies a relative error of r^2 sevenfold (F ~ r^-14) and
// single pair forces can exceed the atom's net force by orders of magnitude;
// the per-atom sums are compensated double-float.  All of this runs on the
// FP32 pipe.  Energy and virial use FP32 terms, summed with compensated FP32
// per thread and FP64 across threads.
#include <cmath>

#include "common.cuh"
#include "lj_impl.cuh"
#include "lj_mixed.cuh"
#include "nlist_impl.cuh"

using namespace mrmd_impl;

namespace mrmd_impl
{
SplitParams split_params(const double* origin, double extent)
{
    SplitParams s{};
    int e = 0;
    std::frexp(extent > 1.0 ? extent : 1.0, &e);  // extent < 2^e
    const int q = 24 - e;
    s = make_split(std::ldexp(1.0, q), std::ldexp(1.0, -q));
    s.origin = make_double3(origin[0], origin[1], origin[2]);
    return s;
}

__global__ void k_split_coords(const double4* __restrict__ pos, int64_t n, SplitParams sp,
                               float4* __restrict__ hi, float4* __restrict__ lo, int stride)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double4 p = pos[i];
        float4 h, l;
        split_one(p.x - sp.origin.x, sp, h.x, l.x);
        split_one(p.y - sp.origin.y, sp, h.y, l.y);
        split_one(p.z - sp.origin.z, sp, h.z, l.z);
        h.w = 0.0f;
        l.w = 0.0f;
        hi[i * stride] = h;
        lo[i * stride] = l;
    }
}

int split_coords(mrmd_ctx* ctx, const double* pos4, int64_t n, const SplitParams& sp, float4* hi, float4* lo,
                 int stride)
{
    if (n == 0) return MRMD_OK;
    k_split_coords<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(reinterpret_cast<const double4*>(pos4), n, sp,
                                                                   hi, lo, stride);
    return after_launch(ctx, "split_coords");
}

namespace
{
constexpr int MX_TB = 128;

struct Acc
{
    df fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, e{0.f, 0.f}, w{0.f, 0.f};

    __device__ __forceinline__ void add(const PairMixed& q)
    {
        df_acc_prod(fx, q.dh.x, q.dl.x, q.ff);
        df_acc_prod(fy, q.dh.y, q.dl.y, q.ff);
        df_acc_prod(fz, q.dh.z, q.dl.z, q.ff);
        df_acc(e, q.e);
        df_acc(w, -0.5f * q.ff.h * q.r2h);
    }

};

template <bool PRED>
__global__ void __launch_bounds__(MX_TB) k_lj_mixed_half(
    const float4* __restrict__ hi, const float4* __restrict__ lo, const double4* __restrict__ pos,
    double* __restrict__ force, const LJDev p, RcSq rc2, const int32_t* __restrict__ counts,
    const int32_t* __restrict__ nbrs, int64_t cap, int64_t n, int64_t begin, int64_t nAll, mrmd_dev::Pred pred,
    double* __restrict__ ev)
{
    __shared__ double red[64];
    Acc acc;
    const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (row < n)
    {
        // list row `row` belongs to particle begin + row (the list's range)
        const int64_t i = begin + row;
        const float4 hi_i = hi[i], lo_i = lo[i];
        double4 pi;
        if (PRED) pi = pos[i];
        const int32_t cnt = counts[row];
        const int32_t* __restrict__ col = nbrs + mrmd_dev::nbr_row(row, cap);
        for (int32_t k = 0; k < cnt; ++k)
        {
            const int32_t j = __ldg(col + 32 * (int64_t)k);
            if (!MRMD_IN_BOUNDS(j, nAll)) continue;
            if (PRED)
            {
                const double4 pj = mrmd_dev::ldg4(pos + j);
                if (!mrmd_dev::pred2(pred, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z)) continue;
            }
            PairMixed q;
            if (!pair_mixed(hi_i, lo_i, __ldg(hi + j), __ldg(lo + j), p, rc2, q)) continue;
            acc.add(q);
            atomicAdd(force + 4 * (int64_t)j + 0, -prod_d(q.dh.x, q.dl.x, q.ff));
            atomicAdd(force + 4 * (int64_t)j + 1, -prod_d(q.dh.y, q.dl.y, q.ff));
            atomicAdd(force + 4 * (int64_t)j + 2, -prod_d(q.dh.z, q.dl.z, q.ff));
        }
        atomicAdd(force + 4 * i + 0, (double)acc.fx.h + (double)acc.fx.l);
        atomicAdd(force + 4 * i + 1, (double)acc.fy.h + (double)acc.fy.l);
        atomicAdd(force + 4 * i + 2, (double)acc.fz.h + (double)acc.fz.l);
    }
    double e = (double)acc.e.h + (double)acc.e.l, w = (double)acc.w.h + (double)acc.w.l;
    mrmd_dev::block_sum2(e, w, red);
    if (threadIdx.x == 0)
    {
        atomicAdd(ev + 0, e);
        atomicAdd(ev + 1, w);
    }
}

}  // namespace

int lj_mixed_half(mrmd_ctx* ctx, const float4* hi, const float4* lo, const mrmd_lj* lj, mrmd_atoms* a,
                  const mrmd_nlist* nl, const mrmd_pred* pred, double* ev)
{
    const int64_t n = nl->rows;
    if (n == 0) return MRMD_OK;
    const bool usePred = pred != nullptr && pred->kind != MRMD_PRED_ALWAYS;
    const unsigned grid = (unsigned)div_up(n, MX_TB);
    const mrmd_dev::Pred dp = to_dev_pred(pred);
    const RcSq rc2 = make_rcsq(lj->rcSqr);
    const double4* pos = reinterpret_cast<const double4*>(a->pos);
    if (usePred)
        k_lj_mixed_half<true><<<grid, MX_TB, 0, ctx->stream>>>(hi, lo, pos, a->force, lj->p0, rc2, nl->counts,
                                                               nl->nbrs, nl->maxNeighbors, n, nl->begin, a->numLocal + a->numGhost, dp, ev);
    else
        k_lj_mixed_half<false><<<grid, MX_TB, 0, ctx->stream>>>(hi, lo, pos, a->force, lj->p0, rc2, nl->counts,
                                                                nl->nbrs, nl->maxNeighbors, n, nl->begin, a->numLocal + a->numGhost, dp, ev);
    return after_launch(ctx, "lj_mixed_half");
}

SplitParams split_params_for(const mrmd_nlist* nl)
{
    const CellList* cl = static_cast<const CellList*>(nl->cells);
    const double origin[3] = {cl->g.mn.x, cl->g.mn.y, cl->g.mn.z};
    return split_params(origin, cl->g.extent * 1.25 + 8.0);
}

int lj_apply_mixed(mrmd_ctx* ctx, const mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl, const mrmd_pred* pred,
                   double* ev)
{
    if (lj->numTypes > 1) return set_error(ctx, MRMD_ERR_ARG, "mixed precision supports one atom type");
    if (nl->rows == 0) return MRMD_OK;
    const SplitParams sp = split_params_for(nl);
    const int64_t nAll = a->numLocal + a->numGhost;
    float4* hi = static_cast<float4*>(scratch(ctx, sizeof(float4) * 2 * (size_t)nAll));
    if (!hi) return MRMD_ERR_OOM;
    float4* lo = hi + nAll;
    MRMD_TRY(split_coords(ctx, a->pos, nAll, sp, hi, lo));
    return lj_mixed_half(ctx, hi, lo, lj, a, nl, pred, ev);
}
}  // namespace mrmd_impl
