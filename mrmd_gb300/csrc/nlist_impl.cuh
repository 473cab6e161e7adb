// Cell grid and cell list shared by the list builder, the atom sort and the
// fused stepper.
#pragma once

#include <vector>

#include "common.cuh"
#include "f32_round.cuh"

namespace mrmd_impl
{
struct CellGrid
{
    double3 mn;   // grid origin
    double3 rdx;  // cells per unit length
    int3 n;       // cells per axis
    int64_t ncell;
    double extent;  // max |coordinate| relative bound used for FP32 error bands
    int reach;      // list builds search cells within +-reach per axis
    float3 mnf, rdxf;  // mn, rdx rounded to FP32 (the binning's FP32 estimate)
};

// n = max(1, floor(L * reach / delta)) cells per axis, edge L/n >= delta / reach,
// so that every pair within delta is within `reach` cells per axis.
CellGrid make_grid(const double* gridMin, const double* gridMax, double delta, int reach = 1);

// cell = clamp(floor((x - min) * rdx), 0, n - 1) per axis, id (ix*ny + iy)*nz + iz.
// A NaN coordinate goes to cell 0: the comparisons are written so that NaN
// fails `t >= 0` (a double-to-int conversion of NaN is not a valid cell).
// Not inlined: the callers reach it only when the FP32 estimate is open.
static __device__ __noinline__ int32_t cell_coord_fp64(double x, double mn, double rdx, int n)
{
    const double t = floor(__dmul_rn(__dsub_rn(x, mn), rdx));
    int c = t >= 0.0 ? (t > (double)(n - 1) ? n - 1 : (int)t) : 0;
    return c;
}

// The same cell as cell_coord_fp64, from the FP32 estimate where it is
// certain (all but a few in ten thousand coordinates): GB300's FP64 pipe
// made the binning kernel FP64 bound.
__device__ __forceinline__ int32_t cell_coord(double x, double mn, double rdx, int n, float mnf, float rdxf)
{
    bool ok;
    const float t = floor_of_scaled(x, mnf, rdxf, &ok);
    if (!ok) return cell_coord_fp64(x, mn, rdx, n);
    return t >= 0.f ? (t > (float)(n - 1) ? n - 1 : (int)t) : 0;
}

__device__ __forceinline__ int32_t cell_of(const double4& p, const CellGrid& g)
{
    const int32_t cx = cell_coord(p.x, g.mn.x, g.rdx.x, g.n.x, g.mnf.x, g.rdxf.x);
    const int32_t cy = cell_coord(p.y, g.mn.y, g.rdx.y, g.n.y, g.mnf.y, g.rdxf.y);
    const int32_t cz = cell_coord(p.z, g.mn.z, g.rdx.z, g.n.z, g.mnf.z, g.rdxf.z);
    return (cx * g.n.y + cy) * g.n.z + cz;
}

__device__ __forceinline__ bool lex_above(const double4& pi, const double4& pj)
{
    return (pj.x > pi.x) || ((pj.x == pi.x) && ((pj.y > pi.y) || ((pj.y == pi.y) && (pj.z > pi.z))));
}

// The candidate spans of particle i in cell ci: the columns within g.reach
// cells per axis (only cell_x >= cell_x(i) for the half list), each column's
// z range [z0, z1] as one contiguous span [s0, s1) of the cell-sorted
// particles.  span(ax, ay, c0, z0, z1, s0, s1) is called in scan order
// (c0: the cell index of (ax, ay, 0)).
template <bool FULL, class Span>
__device__ __forceinline__ void for_each_span(const int32_t* __restrict__ cellStart, const CellGrid& g, int32_t ci,
                                              int64_t nPos, Span&& span)
{
    const int cz = ci % g.n.z;
    const int cy = (ci / g.n.z) % g.n.y;
    const int cx = ci / (g.n.z * g.n.y);
    const int R = g.reach;
    const int axEnd = min(cx + R, g.n.x - 1);
    const int z0 = max(cz - R, 0), z1 = min(cz + R, g.n.z - 1);
    const int ay0 = max(cy - R, 0), ay1 = min(cy + R, g.n.y - 1);
    for (int ax = FULL ? max(cx - R, 0) : cx; ax <= axEnd; ++ax)
    {
        for (int ay = ay0; ay <= ay1; ++ay)
        {
            // cells (ax, ay, z0..z1) are adjacent in the cell order, so their
            // particles form one contiguous span of the sorted arrays
            const int32_t c0 = (ax * g.n.y + ay) * g.n.z;
            const int32_t s0 = cellStart[c0 + z0], s1 = cellStart[c0 + z1 + 1];
            if (!MRMD_IN_BOUNDS(s0, nPos + 1) || !MRMD_IN_BOUNDS(s1, nPos + 1)) continue;
            span(ax, ay, c0, z0, z1, s0, s1);
        }
    }
}

// The candidate test of the list builds: every decision is the FP64
// predicate.  An FP32 prefilter settles the clear cases (outside [rsqLo,
// rsqHi]) and the FP64 positions decide the rest.  FULL: every j != i within
// r; otherwise Cabana's half-neighbour rule (x_j lexicographically above x_i).
// Returns true when j (the candidate q, id in q.w) is kept; d2f: its FP32
// distance squared.
template <bool FULL>
__device__ __forceinline__ bool candidate_kept(const double4* __restrict__ pos, const double4& pi, int64_t i,
                                               float xi, float yi, float zi, const float4& q, double rsq,
                                               float rsqLo, float rsqHi, int64_t nPos, float& d2f)
{
    const int32_t j = __float_as_int(q.w);
    if (j == (int32_t)i || !MRMD_IN_BOUNDS(j, nPos)) return false;
    // lexicographic (x, y, z): float order is exact unless equal
    if (!FULL && q.x < xi) return false;
    const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
    d2f = dx * dx + dy * dy + dz * dz;
    if (d2f > rsqHi) return false;
    if ((FULL || q.x > xi) && d2f < rsqLo) return true;
    const double4 pj = pos[j];
    const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
    return (d2 <= rsq) && (FULL || lex_above(pi, pj));
}

// The candidate scan of the list builds for particle i in cell ci: keep(j,
// d2f) is called for every kept neighbour in scan order.
template <bool FULL, class Keep>
__device__ __forceinline__ void scan_candidates(const double4* __restrict__ pos, const int32_t* __restrict__ cellStart,
                                                const float4* __restrict__ spos, const CellGrid& g, int64_t i,
                                                int32_t ci, double rsq, float rsqLo, float rsqHi, int64_t nPos,
                                                Keep&& keep)
{
    const double4 pi = pos[i];
    const float xi = (float)(pi.x - g.mn.x), yi = (float)(pi.y - g.mn.y), zi = (float)(pi.z - g.mn.z);
    auto candidate = [&](const float4& q) {
        float d2f;
        if (candidate_kept<FULL>(pos, pi, i, xi, yi, zi, q, rsq, rsqLo, rsqHi, nPos, d2f))
            keep(__float_as_int(q.w), d2f);
    };
    for_each_span<FULL>(cellStart, g, ci, nPos, [&](int, int, int32_t, int, int, int32_t s0, int32_t s1) {
        // four candidates loaded per iteration: the loop is bound by the
        // latency of these loads, not by the arithmetic
        int32_t s = s0;
        for (; s + 3 < s1; s += 4)
        {
            const float4 q0 = spos[s], q1 = spos[s + 1], q2 = spos[s + 2], q3 = spos[s + 3];
            candidate(q0);
            candidate(q1);
            candidate(q2);
            candidate(q3);
        }
        for (; s < s1; ++s) candidate(spos[s]);
    });
}

// Particles binned by cell: sorted[] holds particle ids in cell order
// (ascending id inside a cell), spos[] their FP32 coordinates relative to
// the grid origin with the id bit-cast into w.
struct CellList
{
    CellGrid g{};
    int32_t* cellOf = nullptr;
    int32_t* cellStart = nullptr;  // [ncell + 1]
    int32_t* cursor = nullptr;
    int32_t* sorted = nullptr;
    float4* spos = nullptr;
    int64_t capN = 0, capCells = 0, numParticles = 0;

    // morton: order the cells along a Z-order curve instead of row-major (for
    // sorting particles; list builds need the row-major order)
    // nonfinite (device, may be null): set to 1 when a position is NaN or
    // infinite; the caller clears it and reads it at its next sync.
    int build(mrmd_ctx* ctx, const double* pos4, int64_t n, const CellGrid& grid, bool morton = false,
              int32_t* nonfinite = nullptr);
    void release();
};

// full = false: Cabana half list; full = true: every j != i within rlist
// (each pair twice, used by the mixed form so that no j-force is scattered).
int build_half_list(mrmd_ctx* ctx, mrmd_nlist* nl, const double* pos4, int64_t nPos, int64_t begin,
                    int64_t end, double rlist, const CellGrid& grid, int64_t maxNeighbors, bool full);
struct TileList;
// Full list split by distance at build time: pairs closer than rnear (FP32
// distance) in nearList, the rest within rlist in farList; the cell list of
// nearList is used.  Each pair appears in exactly one of the two lists.
// With `tiles` (begin = 0), the lists are built in their tile form
// (lj_tile.cuh) only, in one pass (tile_list_launch); when a tile does not
// fit that pass, the int32 rows are built and their tile form made from them.
// onePass = false: always the int32 rows and then their tile form.
int build_split_list(mrmd_ctx* ctx, mrmd_nlist* nearList, mrmd_nlist* farList, const double* pos4, int64_t nPos,
                     int64_t begin, int64_t end, double rlist, double rnear, const CellGrid& grid,
                     TileList* tiles = nullptr, bool onePass = true);
int list_total_pairs(mrmd_ctx* ctx, mrmd_nlist* nl);
// The tile form of the split full list over rows [0, rows) built in one
// pass from the cell list `cl` (tile_list.cu), without the int32 rows: the
// near/far counts and tl's members and chunks.  flags as build_split_list's;
// flags[4] != 0 when a tile did not fit its tables (the caller then builds
// the int32 rows and their tile form).
int tile_list_launch(mrmd_ctx* ctx, TileList* tl, int64_t rows, int64_t nPos, const CellList& cl, double rsq, float rsqLo, float rsqHi, float nearSqF, mrmd_nlist* nearList,
                     mrmd_nlist* farList, const double* pos4, int32_t* flags);

// MRMD_ERR_ARG unless the list's rows [begin, begin + rows) are particles
// below numLocal and every neighbour index it can hold (the candidates it
// was built over) is below nAll.
int check_list_fits(mrmd_ctx* ctx, const mrmd_nlist* nl, int64_t numLocal, int64_t nAll);
int permute_atoms(mrmd_ctx* ctx, mrmd_atoms* a, mrmd_atoms* shadow, const int32_t* perm, int64_t n);
}  // namespace mrmd_impl
