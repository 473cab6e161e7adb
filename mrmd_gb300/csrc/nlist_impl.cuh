// Cell grid and cell list shared by the list builder, the atom sort and the
// fused stepper.
#pragma once

#include <vector>

#include "common.cuh"

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
};

// n = max(1, floor(L * reach / delta)) cells per axis, edge L/n >= delta / reach,
// so that every pair within delta is within `reach` cells per axis.
CellGrid make_grid(const double* gridMin, const double* gridMax, double delta, int reach = 1);

// cell = clamp(floor((x - min) * rdx), 0, n - 1) per axis, id (ix*ny + iy)*nz + iz.
// A NaN coordinate goes to cell 0: the comparisons are written so that NaN
// fails `t >= 0` (a double-to-int conversion of NaN is not a valid cell).
__device__ __forceinline__ int32_t cell_coord(double x, double mn, double rdx, int n)
{
    const double t = floor(__dmul_rn(__dsub_rn(x, mn), rdx));
    int c = t >= 0.0 ? (t > (double)(n - 1) ? n - 1 : (int)t) : 0;
    return c;
}

__device__ __forceinline__ int32_t cell_of(const double4& p, const CellGrid& g)
{
    const int32_t cx = cell_coord(p.x, g.mn.x, g.rdx.x, g.n.x);
    const int32_t cy = cell_coord(p.y, g.mn.y, g.rdx.y, g.n.y);
    const int32_t cz = cell_coord(p.z, g.mn.z, g.rdx.z, g.n.z);
    return (cx * g.n.y + cy) * g.n.z + cz;
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
// Full list split by distance at build time: pairs closer than rnear (FP32
// distance) in nearList, the rest within rlist in farList; the cell list of
// nearList is used.  Each pair appears in exactly one of the two lists.
int build_split_list(mrmd_ctx* ctx, mrmd_nlist* nearList, mrmd_nlist* farList, const double* pos4, int64_t nPos,
                     int64_t begin, int64_t end, double rlist, double rnear, const CellGrid& grid);
int list_total_pairs(mrmd_ctx* ctx, mrmd_nlist* nl);
// MRMD_ERR_ARG unless the list's rows [begin, begin + rows) are particles
// below numLocal and every neighbour index it can hold (the candidates it
// was built over) is below nAll.
int check_list_fits(mrmd_ctx* ctx, const mrmd_nlist* nl, int64_t numLocal, int64_t nAll);
int permute_atoms(mrmd_ctx* ctx, mrmd_atoms* a, mrmd_atoms* shadow, const int32_t* perm, int64_t n);
}  // namespace mrmd_impl
