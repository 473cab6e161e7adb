// Mixed-form LJ pair force of the fused stepper on shared-memory tiles.
//
// Arithmetic (per pair i, j of the full list, forces written by i only):
// - r^2 as the exact float pair (S + C, err) of lj_tile.cuh.
// - Near rows (pairs closer than r_split + skin/2 at the rebuild) and the rare
//   far-row pair that came closer than r_split: 1/r^2, the LJ force factor
//   u^4 (ff1 u^3 - ff2) and the force products as float pairs (head and
//   first-order error), summed per atom in double-float.
// - Far pairs: one Newton step takes the hardware reciprocal of r^2 to about
//   half an ulp, using the exact low part of r^2; the factor is evaluated in
//   FP32 (|F| <= |F(r_split)| there, 1.16 epsilon/sigma at 1.5 sigma), the
//   forces summed in FP32.
// - Energy and virial: E = ef1 u^6 - ef2 u^3 - shift and -2W = ff1 u^6 - ff2 u^3
//   per uncapped pair (action/LennardJones.hpp:52-78), so the kernel sums
//   u^3, u^6 and the pair count per atom in double-float (these terms are
//   positive: Fast2Sum against a power-of-two offset above any row's sum
//   makes every head addition error-free) and forms E and W once per block
//   in FP64.
//   Capped pairs (inside the capping distance) add their energy and
//   forceFactor * r^2 to separate double-float sums.
// All per-pair work runs on the FP32 pipe: GB300's FP64 rate is a small
// fraction of its FP32 rate, and even the per-atom conversions to FP64 are
// assembled from the float bits with integer operations.
#include <cmath>

#include "common.cuh"
#include "lj_tile.cuh"
#include "nlist_impl.cuh"

using namespace mrmd_impl;

namespace mrmd_impl
{
bool tile_split_params(const double* origin, double extent, double rlist, SplitParams* out)
{
    int e = 0;
    std::frexp(1.0625 * rlist / 2048.0, &e);  // value in [2^(e-1), 2^e)
    const double Q = std::ldexp(1.0, e);      // smallest power of two above it
    if (!(extent + Q < Q * 16777216.0)) return false;
    *out = make_split(1.0 / Q, Q);
    // the records are differences: any origin on the Q grid serves
    // (split_bits takes it as the integer origin / Q; |origin| < 2^40 Q)
    double o[3];
    for (int d = 0; d < 3; ++d)
    {
        o[d] = std::floor(origin[d] / Q) * Q;
        if (!(std::fabs(o[d]) < Q * 1099511627776.0)) return false;
    }
    out->origin = make_double3(o[0], o[1], o[2]);
    out->ko = make_longlong3((long long)(o[0] / Q), (long long)(o[1] / Q), (long long)(o[2] / Q));
    out->q = -e;  // Q = 2^e
    return true;
}

void TileList::release()
{
    dfree(members);
    dfree(memberCount);
    dfree(nearChunks);
    dfree(farChunks);
    members = memberCount = nullptr;
    nearChunks = farChunks = nullptr;
    tilesCap = nearWords = farWords = tiles = 0;
    nearChunksPerRow = farChunksPerRow = 0;
    maxMembers = 0;
    valid = false;
}

TileParams make_tile_params(const LJDev& p, double rcSqr, double rsplit, int64_t farCapacity)
{
    TileParams t{};
    t.p = p;
    t.rc2 = make_rcsq(rcSqr);
    t.rsplitSq = (float)(rsplit * rsplit);
    // Offsets of the u^3 and u^6 sums: a power of two above the largest sum a
    // row can reach, with its pairs no closer than 0.8 sigma (or the capping
    // distance; sigma^6 = ff1 / (2 ff2)) and up to 2 x the far capacity + 64
    // entries.  A pair closer than that (overlapping atoms without a cap) only
    // loses the error-free property of its own addition.
    const double sig2 = p.ff2 > 0.0 ? std::cbrt(p.ff1 / (2.0 * p.ff2)) : 1.0;
    const double rmin2 = std::fmax(p.capSqr, 0.64 * sig2);
    const double u3max = 1.0 / (rmin2 * rmin2 * rmin2);
    const double n = 2.0 * (double)(farCapacity > 0 ? farCapacity : 64) + 64.0;
    int e3 = 0, e6 = 0;
    std::frexp(n * u3max, &e3);
    std::frexp(n * u3max * u3max, &e6);
    t.bias3 = (float)std::ldexp(1.0, e3);
    t.bias6 = (float)std::ldexp(1.0, e6);
    return t;
}
}  // namespace mrmd_impl

namespace
{
constexpr int HT_BITS = 12;
constexpr int HT = 1 << HT_BITS;  // hash slots per tile (load <= TILE_CAP / HT = 0.75)

__global__ void k_tile_split(const double4* __restrict__ pos, int64_t n, SplitParams sp, float4* __restrict__ recA,
                             float2* __restrict__ recB)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        float4 a;
        float2 b;
        tile_split(pos[i], sp, a, b);
        recA[i] = a;
        recB[i] = b;
    }
}

__device__ __forceinline__ uint32_t slot_hash(int32_t j)
{
    return ((uint32_t)j * 2654435761u) >> (32 - HT_BITS);
}

// The tile form of the split full list just built (k_build_list<1, 1>), one
// block per tile of TILE_ROWS rows.  Phase 1 inserts every neighbour index of
// the rows into a shared open-addressing table of the tile's members, phase 2
// numbers the occupied entries in table order (the member slots), phase 3
// rewrites each row as slots in 8-entry chunks.  flags[3]: largest member
// count; flags[4]: a tile did not fit (its chunks stay unwritten; the pair
// kernel then reads the int32 rows); flags[5]: members of all tiles.
__global__ void __launch_bounds__(TILE_ROWS) k_tile_build(
    const int32_t* __restrict__ countsN, const int32_t* __restrict__ nbrsN, int64_t capN,
    const int32_t* __restrict__ countsF, const int32_t* __restrict__ nbrsF, int64_t capF, int64_t rows, int64_t nAll,
    int32_t* __restrict__ flags, int32_t* __restrict__ members, int32_t* __restrict__ memberCount,
    uint4* __restrict__ nearChunks, int64_t chN, uint4* __restrict__ farChunks, int64_t chF)
{
    extern __shared__ int32_t keys[];                         // [HT]
    uint16_t* slot = reinterpret_cast<uint16_t*>(keys + HT);  // [HT]
    __shared__ int32_t warpTot[TILE_ROWS / 32];
    __shared__ int32_t totalS, badS;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t tile = blockIdx.x;
    const int64_t row = tile * TILE_ROWS + tid;
    for (int h = tid; h < HT; h += TILE_ROWS) keys[h] = -1;
    if (tid == 0) badS = 0;
    __syncthreads();

    // most indices are already in the table (a member is the neighbour of
    // about a dozen of the tile's rows): a plain read settles them
    auto insert = [&](int32_t j) {
        if (j < 0 || j >= nAll)
        {
            badS = 1;
            return;
        }
        uint32_t h = slot_hash(j);
        for (int probe = 0; probe < HT; ++probe)
        {
            const int32_t k = keys[h];
            if (k == j) return;
            if (k == -1)
            {
                const int32_t old = atomicCAS(&keys[h], -1, j);
                if (old == -1 || old == j) return;
            }
            h = (h + 1) & (HT - 1);
        }
        badS = 1;  // table full
    };
    int32_t cn = 0, cf = 0;
    const int32_t* colN = nbrsN + mrmd_dev::nbr_row(row, capN);
    const int32_t* colF = nbrsF + mrmd_dev::nbr_row(row, capF);
    if (row < rows)
    {
        cn = countsN[row];
        cf = countsF[row];
        for (int32_t k = 0; k < cn; ++k) insert(colN[32 * (int64_t)k]);
        for (int32_t k = 0; k < cf; ++k) insert(colF[32 * (int64_t)k]);
    }
    __syncthreads();

    // phase 2: slots in table order
    constexpr int PER = HT / TILE_ROWS;
    int32_t local = 0;
    for (int q = 0; q < PER; ++q) local += keys[tid * PER + q] >= 0;
    int32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warpTot[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        int32_t w = lane < TILE_ROWS / 32 ? warpTot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < TILE_ROWS / 32) warpTot[lane] = w;
    }
    __syncthreads();
    int32_t base = (warp > 0 ? warpTot[warp - 1] : 0) + incl - local;
    if (tid == TILE_ROWS - 1) totalS = base + local;
    for (int q = 0; q < PER; ++q)
    {
        const int h = tid * PER + q;
        if (keys[h] >= 0)
        {
            if (base < TILE_CAP)
            {
                slot[h] = (uint16_t)base;
                members[tile * TILE_CAP + base] = keys[h];
            }
            ++base;
        }
    }
    __syncthreads();
    const int32_t total = totalS;
    const bool bad = badS != 0 || total > TILE_CAP;
    if (tid == 0)
    {
        memberCount[tile] = total < TILE_CAP ? total : TILE_CAP;
        atomicMax(&flags[3], total);
        atomicAdd(&flags[5], total);
        if (bad) atomicOr(&flags[4], 1);
    }
    if (bad || row >= rows) return;

    // phase 3: rows as member slots, eight per 16-byte chunk
    auto lookup = [&](int32_t j) -> uint32_t {
        uint32_t h = slot_hash(j);
        for (int probe = 0; probe < HT; ++probe)
        {
            if (keys[h] == j) return slot[h];
            h = (h + 1) & (HT - 1);
        }
        atomicOr(&flags[4], 1);  // unreachable: every kept index was inserted
        return 0u;
    };
    auto write_rows = [&](const int32_t* col, int32_t cnt, uint4* out, int64_t chunks) {
        for (int32_t g0 = 0; g0 < cnt; g0 += 8)
        {
            uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (g0 + q < cnt) w[q >> 1] |= lookup(col[32 * (int64_t)(g0 + q)]) << (16 * (q & 1));
            out[chunk_word(row, g0 >> 3, chunks)] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    };
    write_rows(colN, cn, nearChunks, chN);
    write_rows(colF, cf, farChunks, chF);
}

// ------------------------------------------------------------ pair force --
struct Geom
{
    float dhx, dhy, dhz, dlx, dly, dlz;
    float r2h, r2l;
};

// dh, dl and r^2 = (r2h, r2l) of one pair; false when beyond the cutoff
// (decided on the double-float r^2, so that pairs within 2^-24 of rc^2 land
// on the same side as in FP64).
__device__ __forceinline__ bool pair_geom(const float4& ai, const float2& bi, const float4& aj, const float2& bj,
                                          RcSq rc2, Geom& g)
{
    g.dhx = __fsub_rn(ai.x, aj.x);  // exact
    g.dhy = __fsub_rn(ai.y, aj.y);
    g.dhz = __fsub_rn(ai.z, aj.z);
    g.dlx = __fsub_rn(ai.w, aj.w);
    g.dly = __fsub_rn(bi.x, bj.x);
    g.dlz = __fsub_rn(bi.y, bj.y);
    const float S = __fmaf_rn(g.dhx, g.dhx, __fmaf_rn(g.dhy, g.dhy, __fmul_rn(g.dhz, g.dhz)));  // exact
    // C = sum dl (2 dh + dl)
    const float C = __fmaf_rn(g.dlx, __fmaf_rn(2.0f, g.dhx, g.dlx),
                              __fmaf_rn(g.dly, __fmaf_rn(2.0f, g.dhy, g.dly),
                                        __fmul_rn(g.dlz, __fmaf_rn(2.0f, g.dhz, g.dlz))));
    g.r2h = __fadd_rn(S, C);
    g.r2l = __fsub_rn(C, __fsub_rn(g.r2h, S));
    return !(g.r2h > rc2.h || (g.r2h == rc2.h && g.r2l > rc2.l));
}

struct Sums
{
    float fxh = 0.f, fxl = 0.f, fyh = 0.f, fyl = 0.f, fzh = 0.f, fzl = 0.f;  // double-float pairs
    float gx = 0.f, gy = 0.f, gz = 0.f;    // FP32 pairs
    float s3h, s3l = 0.f, s6h, s6l = 0.f;  // biased sums of u^3, u^6
    int32_t cnt = 0;                       // uncapped pairs in range
    df ec{0.f, 0.f}, wc{0.f, 0.f};         // capped pairs: energy, forceFactor * r^2
};

// s += x for |x| <= bias <= |s| (Fast2Sum: exact error term into the low part)
__device__ __forceinline__ void biased_add(float& sh, float& sl, float x)
{
    const float t = __fadd_rn(sh, x);
    sl = __fadd_rn(sl, __fsub_rn(x, __fsub_rn(t, sh)));
    sh = t;
}

// s += (dh + dl) * (f0 + f1): FMA TwoProd of the head product, first-order
// cross terms and the TwoSum error into the low part (TwoSum, not an offset
// Fast2Sum: a close contact's pair force can exceed any fixed offset)
__device__ __forceinline__ void acc_prod(float& sh, float& sl, float dh, float dl, float f0, float f1)
{
    const float p = __fmul_rn(dh, f0);
    float e = __fmaf_rn(dh, f0, -p);
    e = __fmaf_rn(dh, f1, __fmaf_rn(dl, f0, e));
    const df t = two_sum(sh, p);
    sl = __fadd_rn(sl, __fadd_rn(e, t.l));
    sh = t.h;
}

template <bool CAP>
__device__ __forceinline__ void near_pair(const Geom& g, const TileParams& tp, Sums& s)
{
    float f0, f1;  // forceFactor = f0 + f1
    if (CAP && g.r2h < tp.p.capSqrf)
    {
        // capped branch (action/LennardJones.hpp:68-72): |F| = capCoeff
        const df r2{g.r2h, g.r2l};
        const df dist = df_sqrt(r2);
        const df ff = df_mul(df{tp.p.capCoeff_f, tp.p.capCoeff_l}, df_rcp(dist));
        f0 = ff.h;
        f1 = ff.l;
        const float e = tp.p.eCapShh - (dist.h - tp.p.capDistf) * tp.p.capCoeff_f;
        df_acc(s.ec, e);
        df_acc(s.wc, ff.h * g.r2h);
    }
    else
    {
        // u = 1/r^2 = u0 + u1 (one Newton step on the exact residual), then
        // u^2, u^3, u^4 and forceFactor = u^4 (ff1 u^3 - ff2) as unnormalised
        // float pairs (head, first-order error)
        const float u0 = __fdividef(1.0f, g.r2h);
        const float u1 = __fmul_rn(u0, __fmaf_rn(-g.r2l, u0, __fmaf_rn(-g.r2h, u0, 1.0f)));
        const float p2 = __fmul_rn(u0, u0);
        const float q2 = __fmaf_rn(__fadd_rn(u0, u0), u1, __fmaf_rn(u0, u0, -p2));
        const float p3 = __fmul_rn(p2, u0);
        const float q3 = __fmaf_rn(p2, u1, __fmaf_rn(q2, u0, __fmaf_rn(p2, u0, -p3)));
        const float p4 = __fmul_rn(p2, p2);
        const float q4 = __fmaf_rn(__fadd_rn(p2, p2), q2, __fmaf_rn(p2, p2, -p4));
        const float pa = __fmul_rn(tp.p.ff1h, p3);
        const float qa = __fmaf_rn(tp.p.ff1h, q3, __fmaf_rn(tp.p.ff1l, p3, __fmaf_rn(tp.p.ff1h, p3, -pa)));
        const df ts = two_sum(pa, -tp.p.ff2h);
        const float tl = __fadd_rn(ts.l, __fsub_rn(qa, tp.p.ff2l));
        f0 = __fmul_rn(p4, ts.h);
        f1 = __fmaf_rn(p4, tl, __fmaf_rn(q4, ts.h, __fmaf_rn(p4, ts.h, -f0)));
        // u^3 = p3 + q3 and u^6 = p3^2 + 2 p3 q3 (+ the rounding of p3^2): the
        // head p3 alone carries the seed reciprocal's error, which q3 corrects
        biased_add(s.s3h, s.s3l, p3);
        s.s3l = __fadd_rn(s.s3l, q3);
        const float u6 = __fmul_rn(p3, p3);
        biased_add(s.s6h, s.s6l, u6);
        s.s6l = __fadd_rn(s.s6l, __fmaf_rn(__fadd_rn(p3, p3), q3, __fmaf_rn(p3, p3, -u6)));
        s.cnt += 1;
    }
    acc_prod(s.fxh, s.fxl, g.dhx, g.dlx, f0, f1);
    acc_prod(s.fyh, s.fyl, g.dhy, g.dly, f0, f1);
    acc_prod(s.fzh, s.fzl, g.dhz, g.dlz, f0, f1);
}

__device__ __forceinline__ void far_pair(const Geom& g, const TileParams& tp, Sums& s)
{
    float u = __fdividef(1.0f, g.r2h);
    u = __fmaf_rn(u, __fmaf_rn(-g.r2l, u, __fmaf_rn(-g.r2h, u, 1.0f)), u);
    const float u2 = __fmul_rn(u, u);
    const float u3 = __fmul_rn(u2, u);
    const float u4 = __fmul_rn(u2, u2);
    // forceFactor = u^3 (ff1 u^3 - ff2) u (action/LennardJones.hpp:60-66)
    const float ff = __fmul_rn(u4, __fmaf_rn(tp.p.ff1h, u3, -tp.p.ff2h));
    s.gx = __fmaf_rn(__fadd_rn(g.dhx, g.dlx), ff, s.gx);
    s.gy = __fmaf_rn(__fadd_rn(g.dhy, g.dly), ff, s.gy);
    s.gz = __fmaf_rn(__fadd_rn(g.dhz, g.dlz), ff, s.gz);
    biased_add(s.s3h, s.s3l, u3);
    biased_add(s.s6h, s.s6l, __fmul_rn(u3, u3));
    s.cnt += 1;
}

// The double with the value of a normal FP32 number (or zero), assembled
// from its bits with integer operations: GB300 runs FP64 conversions on its
// small FP64 pipe.  Subnormal inputs become zero, Inf / NaN keep their class.
__device__ __forceinline__ double f32_as_f64(float x)
{
    const uint32_t b = __float_as_uint(x);
    const uint32_t e = (b >> 23) & 0xffu;
    const uint32_t sign = b & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    const uint32_t de = e == 0xffu ? 0x7ffu : e + 896u;
    return __hiloint2double((int)(sign | (de << 20) | ((b >> 3) & 0xfffffu)), (int)(b << 29));
}

// (h + l) as a double: one FP64 addition of two exact conversions
__device__ __forceinline__ double df_as_f64(float h, float l) { return __dadd_rn(f32_as_f64(h), f32_as_f64(l)); }

__device__ __forceinline__ df shfl_down_df(df v, int o)
{
    return df{__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
}

// Neighbour records of slot / index `idx`.
template <bool TILE>
__device__ __forceinline__ void load_rec(const float4* __restrict__ shA, const float2* __restrict__ shB,
                                         const float4* __restrict__ recA, const float2* __restrict__ recB,
                                         int32_t idx, float4& a, float2& b)
{
    if (TILE)
    {
        a = shA[idx];
        b = shB[idx];
    }
    else
    {
        a = __ldg(recA + idx);
        b = __ldg(recB + idx);
    }
}

// TILE: one block per tile, rows as 16-bit member slots in 8-entry chunks
// (capN, capF: chunks per row), member records in shared memory; otherwise
// rows as int32 particle indices (capN, capF: list capacities), records
// gathered from global memory (fallback and comparison form).
template <bool TILE, bool CAP>
__global__ void __launch_bounds__(TILE_ROWS, 4) k_lj_tile(
    const float4* __restrict__ recA, const float2* __restrict__ recB, const int32_t* __restrict__ members,
    const int32_t* __restrict__ memberCount, int32_t smemStride, const int32_t* __restrict__ countsN,
    const void* __restrict__ colsN, int64_t capN, const int32_t* __restrict__ countsF,
    const void* __restrict__ colsF, int64_t capF, int64_t rows, int64_t nAll, double4* __restrict__ force,
    const TileParams tp, double* __restrict__ ev)
{
    extern __shared__ float4 smem[];
    float4* shA = smem;
    float2* shB = reinterpret_cast<float2*>(smem + smemStride);
    __shared__ float red[TILE_ROWS / 32][10];
    const int tid = threadIdx.x;
    const int64_t tile = blockIdx.x;
    int32_t nMem = 0;
    if (TILE)
    {
        nMem = memberCount[tile];
        const int32_t* mem = members + tile * TILE_CAP;
        for (int32_t t = tid; t < nMem; t += TILE_ROWS)
        {
            const int32_t j = mem[t];
            if (!MRMD_IN_BOUNDS(j, nAll)) continue;
            shA[t] = __ldg(recA + j);
            shB[t] = __ldg(recB + j);
        }
        __syncthreads();
    }
    const int64_t row = tile * TILE_ROWS + tid;
    const int32_t bound = TILE ? nMem : (int32_t)nAll;
    (void)bound;  // read by MRMD_IN_BOUNDS in the bounds-checked build
    Sums s;
    s.s3h = tp.bias3;
    s.s6h = tp.bias6;
    if (row < rows)
    {
        const float4 ai = __ldg(recA + row);
        const float2 bi = __ldg(recB + row);
        const int32_t cn = countsN[row], cf = countsF[row];
        // one pair of slot (TILE) or particle index `idx`: near rows always in
        // double-float, far rows in FP32 unless the pair came within r_split
        auto pair = [&](int32_t idx, bool nearRow) {
            if (!MRMD_IN_BOUNDS(idx, bound)) return;
            float4 aj;
            float2 bj;
            load_rec<TILE>(shA, shB, recA, recB, idx, aj, bj);
            Geom g;
            if (!pair_geom(ai, bi, aj, bj, tp.rc2, g)) return;
            if (nearRow || g.r2h < tp.rsplitSq)
                near_pair<CAP>(g, tp, s);
            else
                far_pair(g, tp, s);
        };
        if (TILE)
        {
            // eight slots per 16-byte chunk load
            auto rows_of = [&](const uint4* __restrict__ chunks, int64_t nch, int32_t cnt, bool nearRow) {
                const int64_t base = chunk_word(row, 0, nch);
                for (int32_t g0 = 0; g0 < cnt; g0 += 8)
                {
                    const uint4 c = __ldg(chunks + base + ((int64_t)(g0 >> 3) << 5));
                    uint64_t lo = ((uint64_t)c.y << 32) | c.x, hi = ((uint64_t)c.w << 32) | c.z;
                    const int32_t m = cnt - g0 < 8 ? cnt - g0 : 8;
                    for (int32_t q = 0; q < m; ++q)
                    {
                        const int32_t idx = (int32_t)(lo & 0xffffu);
                        lo = (lo >> 16) | (hi << 48);
                        hi >>= 16;
                        pair(idx, nearRow);
                    }
                }
            };
            rows_of(static_cast<const uint4*>(colsN), capN, cn, true);
            rows_of(static_cast<const uint4*>(colsF), capF, cf, false);
        }
        else
        {
            const int32_t* __restrict__ nI = static_cast<const int32_t*>(colsN) + mrmd_dev::nbr_row(row, capN);
            const int32_t* __restrict__ fI = static_cast<const int32_t*>(colsF) + mrmd_dev::nbr_row(row, capF);
#pragma unroll 2
            for (int32_t k = 0; k < cn; ++k) pair(__ldg(nI + 32 * (int64_t)k), true);
#pragma unroll 2
            for (int32_t k = 0; k < cf; ++k) pair(__ldg(fI + 32 * (int64_t)k), false);
        }
        // F = near double-float sum + far FP32 sum
        auto comp = [&](float h, float l, float gsum) -> double {
            const df t = two_sum(h, gsum);
            return df_as_f64(t.h, __fadd_rn(t.l, l));
        };
        force[row] = make_double4(comp(s.fxh, s.fxl, s.gx), comp(s.fyh, s.fyl, s.gy), comp(s.fzh, s.fzl, s.gz), 0.0);
    }
    // per-thread sums without the offsets (exact: the heads lie in
    // [bias, 2 bias)), then a double-float block reduction on the FP32 pipe
    df v[5] = {fast_two_sum(__fsub_rn(s.s3h, tp.bias3), s.s3l), fast_two_sum(__fsub_rn(s.s6h, tp.bias6), s.s6l),
               df{(float)s.cnt, 0.f}, s.ec, s.wc};
    const int nv = CAP ? 5 : 3;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < 5; ++q)
            if (q < nv) v[q] = df_add(v[q], shfl_down_df(v[q], o));
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 5; ++q)
        {
            red[warp][2 * q] = v[q].h;
            red[warp][2 * q + 1] = v[q].l;
        }
    __syncthreads();
    if (warp == 0)
    {
#pragma unroll
        for (int q = 0; q < 5; ++q)
            v[q] = lane < TILE_ROWS / 32 ? df{red[lane][2 * q], red[lane][2 * q + 1]} : df{0.f, 0.f};
#pragma unroll
        for (int o = TILE_ROWS / 64; o > 0; o >>= 1)
#pragma unroll
            for (int q = 0; q < 5; ++q)
                if (q < nv) v[q] = df_add(v[q], shfl_down_df(v[q], o));
        if (lane == 0)
        {
            const double s3 = df_as_f64(v[0].h, v[0].l), s6 = df_as_f64(v[1].h, v[1].l);
            const double c = df_as_f64(v[2].h, v[2].l);
            const double ec = CAP ? df_as_f64(v[3].h, v[3].l) : 0.0, wc = CAP ? df_as_f64(v[4].h, v[4].l) : 0.0;
            // every pair appears in both rows: halve
            const double e = 0.5 * (tp.p.ef1 * s6 - tp.p.ef2 * s3 - tp.p.shift * c + ec);
            const double w = -0.25 * (tp.p.ff1 * s6 - tp.p.ff2 * s3 + wc);
            atomicAdd(ev + 0, e);
            atomicAdd(ev + 1, w);
        }
    }
}
}  // namespace

namespace mrmd_impl
{
int tile_split_coords(mrmd_ctx* ctx, const double* pos4, int64_t n, const SplitParams& sp, float4* recA,
                      float2* recB)
{
    if (n == 0) return MRMD_OK;
    k_tile_split<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(reinterpret_cast<const double4*>(pos4), n, sp,
                                                                 recA, recB);
    return after_launch(ctx, "tile_split");
}

int tile_storage(mrmd_ctx* ctx, TileList* tl, int64_t rows, int64_t capN, int64_t capF)
{
    tl->valid = false;
    tl->tiles = div_up(rows, TILE_ROWS);
    if (tl->tiles > tl->tilesCap)
    {
        dfree(tl->members);
        dfree(tl->memberCount);
        tl->members = tl->memberCount = nullptr;
        const int64_t c = tl->tiles + tl->tiles / 8 + 4;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&tl->members), sizeof(int32_t) * (size_t)c * TILE_CAP));
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&tl->memberCount), sizeof(int32_t) * (size_t)c));
        tl->tilesCap = c;
    }
    tl->nearChunksPerRow = div_up(capN, 8);
    tl->farChunksPerRow = div_up(capF, 8);
    const int64_t rows32 = div_up(rows, 32) * 32;
    if (rows32 * tl->nearChunksPerRow > tl->nearWords)
    {
        dfree(tl->nearChunks);
        tl->nearChunks = nullptr;
        const int64_t w = rows32 * tl->nearChunksPerRow + rows32 * tl->nearChunksPerRow / 8;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&tl->nearChunks), sizeof(uint4) * (size_t)w));
        tl->nearWords = w;
    }
    if (rows32 * tl->farChunksPerRow > tl->farWords)
    {
        dfree(tl->farChunks);
        tl->farChunks = nullptr;
        const int64_t w = rows32 * tl->farChunksPerRow + rows32 * tl->farChunksPerRow / 8;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&tl->farChunks), sizeof(uint4) * (size_t)w));
        tl->farWords = w;
    }
    // the pair kernel's shared-memory limit (per device; set here, outside
    // any stream capture)
    const int maxPair = TILE_CAP * (int)(sizeof(float4) + sizeof(float2));
    MRMD_CUDA(ctx, cudaFuncSetAttribute(k_lj_tile<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxPair));
    MRMD_CUDA(ctx, cudaFuncSetAttribute(k_lj_tile<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxPair));
    return MRMD_OK;
}

int tile_build_launch(mrmd_ctx* ctx, TileList* tl, int64_t rows, int64_t nAll, const mrmd_nlist* nearList,
                      const mrmd_nlist* farList, int32_t* flags)
{
    const int64_t capN = nearList->maxNeighbors, capF = farList->maxNeighbors;
    MRMD_TRY(tile_storage(ctx, tl, rows, capN, capF));
    if (rows == 0) return MRMD_OK;
    const size_t smem = sizeof(int32_t) * HT + sizeof(uint16_t) * HT;
    k_tile_build<<<(unsigned)tl->tiles, TILE_ROWS, smem, ctx->stream>>>(
        nearList->counts, nearList->nbrs, capN, farList->counts, farList->nbrs, capF, rows, nAll, flags, tl->members,
        tl->memberCount, tl->nearChunks, tl->nearChunksPerRow, tl->farChunks, tl->farChunksPerRow);
    return after_launch(ctx, "tile_build");
}

void tile_build_done(TileList* tl, int32_t maxMembers, bool valid, int64_t totalMembers)
{
    tl->maxMembers = maxMembers;
    tl->valid = valid;
    tl->totalMembers = totalMembers;
}

int lj_tile_forces(mrmd_ctx* ctx, const TileList* tl, const mrmd_nlist* nearList, const mrmd_nlist* farList,
                   const float4* recA, const float2* recB, double* force4, const TileParams& tp, double* ev,
                   int64_t nAll, bool gather)
{
    const int64_t rows = nearList->rows;
    if (rows == 0) return MRMD_OK;
    const unsigned grid = (unsigned)div_up(rows, TILE_ROWS);
    const bool cap = tp.p.capSqr > 0.0;
    double4* f = reinterpret_cast<double4*>(force4);
    if (tl && tl->valid && !gather)
    {
        // members of the largest tile, rounded to 16 (shB starts 16-byte aligned)
        const int32_t stride = (int32_t)((tl->maxMembers + 15) / 16 * 16);
        const size_t smem = (size_t)stride * (sizeof(float4) + sizeof(float2));
#define TILE_LAUNCH(CAPV)                                                                                          \
    k_lj_tile<true, CAPV><<<grid, TILE_ROWS, smem, ctx->stream>>>(                                                \
        recA, recB, tl->members, tl->memberCount, stride, nearList->counts, tl->nearChunks, tl->nearChunksPerRow,  \
        farList->counts, tl->farChunks, tl->farChunksPerRow, rows, nAll, f, tp, ev)
        if (cap)
            TILE_LAUNCH(true);
        else
            TILE_LAUNCH(false);
#undef TILE_LAUNCH
        return after_launch(ctx, "lj_tile");
    }
#define GATHER_LAUNCH(CAPV)                                                                                        \
    k_lj_tile<false, CAPV><<<grid, TILE_ROWS, 0, ctx->stream>>>(                                                  \
        recA, recB, nullptr, nullptr, 0, nearList->counts, nearList->nbrs, nearList->maxNeighbors, farList->counts, \
        farList->nbrs, farList->maxNeighbors, rows, nAll, f, tp, ev)
    if (cap)
        GATHER_LAUNCH(true);
    else
        GATHER_LAUNCH(false);
#undef GATHER_LAUNCH
    return after_launch(ctx, "lj_tile_gather");
}
}  // namespace mrmd_impl
