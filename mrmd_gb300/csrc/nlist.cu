// Linked cells and the half Verlet list (Cabana::LinkedCellList +
// Cabana::VerletList<HalfNeighborTag, VerletLayout2D> as used by MRMD).
//
// Pair rule (Cabana 0.7, NeighborDiscriminator<HalfNeighborTag>): particle
// j is a neighbour of i when j != i, |x_i - x_j|^2 <= r^2 and x_j is above
// x_i in lexicographic (x, y, z) order.  Every test below decides exactly
// the FP64 predicate: an FP32 prefilter settles the clear cases and the
// FP64 positions decide everything inside the FP32 error band, so the pair
// set is bit-identical to an all-FP64 build.
//
// Because x_j >= x_i implies cell_x(j) >= cell_x(i) (floor is monotone),
// only the 9 + 9 cells with cell_x >= cell_x(i) can hold neighbours.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "nlist_impl.cuh"
#include "lj_tile.cuh"

using namespace mrmd_impl;

namespace mrmd_impl
{
CellGrid make_grid(const double* gridMin, const double* gridMax, double delta, int reach)
{
    // n = max(1, floor(L reach / delta)) cells per axis, edge L / n >= delta / reach
    CellGrid g{};
    g.reach = reach < 1 ? 1 : reach;
    delta /= g.reach;
    double mn[3], rdx[3];
    int n[3];
    double extent = 0.0;
    for (int d = 0; d < 3; ++d)
    {
        const double L = gridMax[d] - gridMin[d];
        int64_t c = (int64_t)std::floor(L / delta);
        if (c < 1) c = 1;
        n[d] = (int)c;
        mn[d] = gridMin[d];
        rdx[d] = (double)c / L;
        extent = std::fmax(extent, std::fmax(std::fabs(gridMin[d]), std::fabs(gridMax[d])));
        extent = std::fmax(extent, L);
    }
    g.mn = make_double3(mn[0], mn[1], mn[2]);
    g.rdx = make_double3(rdx[0], rdx[1], rdx[2]);
    g.mnf = make_float3((float)mn[0], (float)mn[1], (float)mn[2]);
    g.rdxf = make_float3((float)rdx[0], (float)rdx[1], (float)rdx[2]);
    g.n = make_int3(n[0], n[1], n[2]);
    g.ncell = (int64_t)n[0] * n[1] * n[2];
    g.extent = extent;
    return g;
}

// Bits of v spread to every third position (v < 2^10).
__device__ __forceinline__ uint32_t spread3(uint32_t v)
{
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// morton != 0: the key is the Morton (Z-order) code of the cell coordinates,
// so that particles sorted by it form compact blocks in space.
// nonfinite (may be null): set to 1 when a position is NaN or infinite (such
// a particle is binned into a clamped cell and never becomes a neighbour).
__global__ void k_cell_count(const double4* __restrict__ pos, int64_t n, CellGrid g,
                             int32_t* __restrict__ cellOf, int32_t* __restrict__ cellCount, int morton,
                             int32_t* __restrict__ nonfinite, int64_t nkeys)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        int32_t c;
        const double4 p = pos[i];
        // finite: exponent field below all ones (integer test, no FP64 compare)
        const uint32_t ex = (uint32_t)(__double_as_longlong(p.x) >> 52) & 0x7ffu;
        const uint32_t ey = (uint32_t)(__double_as_longlong(p.y) >> 52) & 0x7ffu;
        const uint32_t ez = (uint32_t)(__double_as_longlong(p.z) >> 52) & 0x7ffu;
        if (nonfinite && (ex == 0x7ffu || ey == 0x7ffu || ez == 0x7ffu)) *nonfinite = 1;
        if (morton)
        {
            const uint32_t cx = (uint32_t)cell_coord(p.x, g.mn.x, g.rdx.x, g.n.x, g.mnf.x, g.rdxf.x);
            const uint32_t cy = (uint32_t)cell_coord(p.y, g.mn.y, g.rdx.y, g.n.y, g.mnf.y, g.rdxf.y);
            const uint32_t cz = (uint32_t)cell_coord(p.z, g.mn.z, g.rdx.z, g.n.z, g.mnf.z, g.rdxf.z);
            c = (int32_t)((spread3(cx) << 2) | (spread3(cy) << 1) | spread3(cz));
        }
        else
        {
            c = cell_of(p, g);
        }
        cellOf[i] = c;
        if (MRMD_IN_BOUNDS(c, nkeys)) atomicAdd(&cellCount[c], 1);
    }
}

__global__ void k_cell_scatter(const int32_t* __restrict__ cellOf, int64_t n,
                               const int32_t* __restrict__ cellStart, int32_t* __restrict__ cursor,
                               int32_t* __restrict__ sorted, int64_t nkeys)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t c = cellOf[i];
        if (!MRMD_IN_BOUNDS(c, nkeys)) continue;
        const int64_t slot = cellStart[c] + atomicAdd(&cursor[c], 1);
        if (MRMD_IN_BOUNDS(slot, n)) sorted[slot] = (int32_t)i;
    }
}

// Stable order inside each cell: every slot of the (unordered) scatter
// output counts the smaller ids of its cell and moves its id to that rank.
__global__ void k_cell_rank(const int32_t* __restrict__ cellOf, const int32_t* __restrict__ cellStart,
                            const int32_t* __restrict__ unordered, int64_t n, int32_t* __restrict__ sorted,
                            int64_t nkeys)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t v = unordered[s];
        if (!MRMD_IN_BOUNDS(v, n)) continue;
        const int32_t c = cellOf[v];
        if (!MRMD_IN_BOUNDS(c, nkeys)) continue;
        const int32_t b = cellStart[c], e = cellStart[c + 1];
        if (!MRMD_IN_BOUNDS(b, n + 1) || !MRMD_IN_BOUNDS(e, n + 1)) continue;
        int32_t rank = 0;
        for (int32_t t = b; t < e; ++t) rank += unordered[t] < v;
        if (MRMD_IN_BOUNDS(b + rank, n)) sorted[b + rank] = v;
    }
}

__global__ void k_cell_gather(const double4* __restrict__ pos, const int32_t* __restrict__ sorted,
                              int64_t n, double3 origin, float4* __restrict__ spos)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t j = sorted[s];
        if (!MRMD_IN_BOUNDS(j, n)) continue;
        const double4 p = pos[j];
        spos[s] = make_float4((float)(p.x - origin.x), (float)(p.y - origin.y), (float)(p.z - origin.z),
                              __int_as_float(j));
    }
}

// SPLIT (full lists only): pairs with an FP32 distance below sqrt(nearSqF)
// go to the first list, the others to the second (`capFar`, `countsFar`,
// `nbrsFar`, overflow in maxCount[1]).  The split is a placement choice, not
// a cutoff: every kept pair is in exactly one of the two lists.
template <bool FULL, bool SPLIT = false>
__global__ void __launch_bounds__(128) k_build_list(
    const double4* __restrict__ pos, const int32_t* __restrict__ cellOf,
    const int32_t* __restrict__ cellStart, const float4* __restrict__ spos, CellGrid g,
    int64_t begin, int64_t end, double rsq, float rsqLo, float rsqHi, int64_t cap,
    int32_t* __restrict__ counts, int32_t* __restrict__ nbrs, int32_t* __restrict__ maxCount, int64_t nPos,
    float nearSqF = 0.0f, int64_t capFar = 0, int32_t* __restrict__ countsFar = nullptr,
    int32_t* __restrict__ nbrsFar = nullptr)
{
    for (int64_t i = begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < end;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t ci = cellOf[i];
        if (!MRMD_IN_BOUNDS(ci, g.ncell)) continue;
        int32_t cnt = 0, cntFar = 0;
        const int64_t row = i - begin;
        scan_candidates<FULL>(pos, cellStart, spos, g, i, ci, rsq, rsqLo, rsqHi, nPos, [&](int32_t j, float d2f) {
            if (SPLIT && d2f >= nearSqF)
            {
                if (cntFar < capFar) nbrsFar[mrmd_dev::nbr_row(row, capFar) + 32 * (int64_t)cntFar] = j;
                ++cntFar;
                return;
            }
            if (cnt < cap) nbrs[mrmd_dev::nbr_row(row, cap) + 32 * (int64_t)cnt] = j;
            ++cnt;
        });
        counts[row] = cnt < cap ? cnt : (int32_t)cap;
        if (cnt > cap) atomicMax(maxCount, cnt);
        if (SPLIT)
        {
            countsFar[row] = cntFar < capFar ? cntFar : (int32_t)capFar;
            if (cntFar > capFar) atomicMax(maxCount + 1, cntFar);
        }
    }
}

int CellList::build(mrmd_ctx* ctx, const double* pos4, int64_t n, const CellGrid& grid, bool morton,
                    int32_t* nonfinite)
{
    g = grid;
    // Morton keys need at most 10 bits per axis; the key range is then a
    // power-of-two cube covering the grid
    int bits = 0;
    while ((1 << bits) < std::max(g.n.x, std::max(g.n.y, g.n.z))) ++bits;
    if (bits > 10) morton = false;
    const int64_t nkeys = morton ? (int64_t)1 << (3 * bits) : g.ncell;
    if (n > INT32_MAX || g.ncell > INT32_MAX) return set_error(ctx, MRMD_ERR_CAPACITY, "too many particles or cells");
    if (n + 1 > capN)
    {
        dfree(cellOf);
        dfree(sorted);
        dfree(spos);
        cellOf = sorted = nullptr;
        spos = nullptr;
        const int64_t c = n + n / 4 + 64;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&cellOf), sizeof(int32_t) * (size_t)c));
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&sorted), sizeof(int32_t) * (size_t)c));
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&spos), sizeof(float4) * (size_t)c));
        capN = c;
    }
    if (nkeys + 1 > capCells)
    {
        dfree(cellStart);
        dfree(cursor);
        cellStart = cursor = nullptr;
        const int64_t c = nkeys + 1;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&cellStart), sizeof(int32_t) * (size_t)c));
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&cursor), sizeof(int32_t) * (size_t)c));
        capCells = c;
    }
    numParticles = n;
    constexpr int TB = 256;
    MRMD_CUDA(ctx, cudaMemsetAsync(cellStart, 0, sizeof(int32_t) * (size_t)(nkeys + 1), ctx->stream));
    MRMD_CUDA(ctx, cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)(nkeys + 1), ctx->stream));
    if (n > 0)
    {
        k_cell_count<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(pos4), n,
                                                                   g, cellOf, cellStart, morton ? 1 : 0,
                                                                   nonfinite, nkeys);
        MRMD_TRY(after_launch(ctx, "cell_count"));
    }
    MRMD_TRY(scan_exclusive_i32(ctx, cellStart, cellStart, nkeys + 1, nullptr));
    if (n > 0)
    {
        // unordered scatter into `spos` storage (reused as int32 scratch), then
        // stable ranks into `sorted`
        int32_t* unordered = reinterpret_cast<int32_t*>(spos);
        k_cell_scatter<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(cellOf, n, cellStart, cursor, unordered, nkeys);
        MRMD_TRY(after_launch(ctx, "cell_scatter"));
        k_cell_rank<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(cellOf, cellStart, unordered, n, sorted, nkeys);
        MRMD_TRY(after_launch(ctx, "cell_rank"));
        k_cell_gather<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(pos4),
                                                                    sorted, n, g.mn, spos);
        MRMD_TRY(after_launch(ctx, "cell_gather"));
    }
    return MRMD_OK;
}

void CellList::release()
{
    dfree(cellOf);
    dfree(sorted);
    dfree(spos);
    dfree(cellStart);
    dfree(cursor);
    cellOf = sorted = cellStart = cursor = nullptr;
    spos = nullptr;
    capN = capCells = 0;
}

static int ensure_list_storage(mrmd_ctx* ctx, mrmd_nlist* nl, int64_t rows, int64_t maxNeighbors)
{
    const int64_t stride = div_up(rows > 0 ? rows : 1, 32) * 32;
    if (rows + 1 > nl->rowsCapacity)
    {
        dfree(nl->counts);
        nl->counts = nullptr;
        const int64_t c = rows + rows / 8 + 64;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&nl->counts), sizeof(int32_t) * (size_t)c));
        nl->rowsCapacity = c;
    }
    const int64_t need = stride * maxNeighbors;
    if (need > nl->nbrsCapacity)
    {
        dfree(nl->nbrs);
        nl->nbrs = nullptr;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&nl->nbrs), sizeof(int32_t) * (size_t)need));
        nl->nbrsCapacity = need;
    }
    nl->stride = 32;  // slot step inside a 32-row tile
    nl->maxNeighbors = maxNeighbors;
    return MRMD_OK;
}

int build_half_list(mrmd_ctx* ctx, mrmd_nlist* nl, const double* pos4, int64_t nPos, int64_t begin,
                    int64_t end, double rlist, const CellGrid& grid, int64_t maxNeighbors, bool full)
{
    CellList* cl = static_cast<CellList*>(nl->cells);
    // [0] longest row, [2] non-finite position flag
    int32_t* maxCount = reinterpret_cast<int32_t*>(ctx->devScalars);
    MRMD_CUDA(ctx, cudaMemsetAsync(maxCount, 0, 3 * sizeof(int32_t), ctx->stream));
    MRMD_TRY(cl->build(ctx, pos4, nPos, grid, false, maxCount + 2));
    const int64_t rows = end - begin;
    // FP32 error band: coordinates are stored relative to the grid origin
    // (|c| <= extent), each rounding error <= 2^-24 |c|, so |dx_f - dx| <=
    // delta := 2^-22 extent and |d2_f - d2| <= 6 r delta + 3 delta^2 plus the
    // FP32 rounding of the sum (< 2^-21 d2).
    const double delta = std::ldexp(grid.extent, -22);
    const double band = 6.0 * rlist * delta + 3.0 * delta * delta + std::ldexp(rlist * rlist, -20);
    const double rsq = rlist * rlist;
    const float rsqLo = (float)std::fmax(0.0, (rsq - 2.0 * band) * (1.0 - 1e-6));
    const float rsqHi = (float)((rsq + 2.0 * band) * (1.0 + 1e-6));
    int64_t cap = maxNeighbors > 0 ? maxNeighbors : 64;
    for (int attempt = 0; attempt < 4; ++attempt)
    {
        MRMD_TRY(ensure_list_storage(ctx, nl, rows, cap));
        MRMD_CUDA(ctx, cudaMemsetAsync(maxCount, 0, sizeof(int32_t), ctx->stream));
        if (rows > 0)
        {
            if (full)
                k_build_list<true><<<grid_for(ctx, rows, 128, 16), 128, 0, ctx->stream>>>(
                    reinterpret_cast<const double4*>(pos4), cl->cellOf, cl->cellStart, cl->spos, cl->g, begin,
                    end, rsq, rsqLo, rsqHi, cap, nl->counts, nl->nbrs, maxCount, nPos);
            else
                k_build_list<false><<<grid_for(ctx, rows, 128, 16), 128, 0, ctx->stream>>>(
                    reinterpret_cast<const double4*>(pos4), cl->cellOf, cl->cellStart, cl->spos, cl->g, begin,
                    end, rsq, rsqLo, rsqHi, cap, nl->counts, nl->nbrs, maxCount, nPos);
            MRMD_TRY(after_launch(ctx, "build_list"));
        }
        int32_t h[3] = {0, 0, 0};
        MRMD_CUDA(ctx, cudaMemcpyAsync(h, maxCount, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        MRMD_TRY(bounds_check(ctx));
        if (h[2]) return set_error(ctx, MRMD_ERR_NONFINITE, "non-finite particle position at the list build");
        const int32_t hMax = h[0];
        if (hMax <= cap)
        {
            nl->rows = rows;
            nl->begin = begin;
            return MRMD_OK;
        }
        cap = hMax + hMax / 8 + 4;  // Cabana grows and rebuilds the same way
    }
    return set_error(ctx, MRMD_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
}

__global__ void k_count_sum(const int32_t* __restrict__ counts, int64_t n, unsigned long long* out)
{
    unsigned long long s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)counts[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

int build_split_list(mrmd_ctx* ctx, mrmd_nlist* nearList, mrmd_nlist* farList, const double* pos4, int64_t nPos,
                     int64_t begin, int64_t end, double rlist, double rnear, const CellGrid& grid, TileList* tiles,
                     bool onePass)
{
    if (tiles && begin != 0) return set_error(ctx, MRMD_ERR_ARG, "tile lists need rows from particle 0");
    CellList* cl = static_cast<CellList*>(nearList->cells);
    // [0], [1] longest near and far rows, [2] non-finite position flag
    int32_t* maxCount = reinterpret_cast<int32_t*>(ctx->devScalars);
    MRMD_CUDA(ctx, cudaMemsetAsync(maxCount, 0, 3 * sizeof(int32_t), ctx->stream));
    MRMD_TRY(cl->build(ctx, pos4, nPos, grid, false, maxCount + 2));
    const int64_t rows = end - begin;
    // the same FP32 error band as build_half_list
    const double delta = std::ldexp(grid.extent, -22);
    const double band = 6.0 * rlist * delta + 3.0 * delta * delta + std::ldexp(rlist * rlist, -20);
    const double rsq = rlist * rlist;
    const float rsqLo = (float)std::fmax(0.0, (rsq - 2.0 * band) * (1.0 - 1e-6));
    const float rsqHi = (float)((rsq + 2.0 * band) * (1.0 + 1e-6));
    const float nearSqF = (float)(rnear * rnear);
    int64_t capN = nearList->maxNeighbors > 0 ? nearList->maxNeighbors : 32;
    int64_t capF = farList->maxNeighbors > 0 ? farList->maxNeighbors : 64;
    for (int attempt = 0; attempt < 4; ++attempt)
    {
        MRMD_TRY(ensure_list_storage(ctx, nearList, rows, capN));
        MRMD_TRY(ensure_list_storage(ctx, farList, rows, capF));
        // [3..5]: the tile build's largest tile, overflow flag, member total
        MRMD_CUDA(ctx, cudaMemsetAsync(maxCount, 0, 2 * sizeof(int32_t), ctx->stream));
        MRMD_CUDA(ctx, cudaMemsetAsync(maxCount + 3, 0, 3 * sizeof(int32_t), ctx->stream));
        auto int32_rows = [&]() -> int {
            k_build_list<true, true><<<grid_for(ctx, rows, 128, 16), 128, 0, ctx->stream>>>(
                reinterpret_cast<const double4*>(pos4), cl->cellOf, cl->cellStart, cl->spos, cl->g, begin, end,
                rsq, rsqLo, rsqHi, capN, nearList->counts, nearList->nbrs, maxCount, nPos, nearSqF, capF,
                farList->counts, farList->nbrs);
            return after_launch(ctx, "build_split_list");
        };
        if (rows > 0)
        {
            if (tiles && !onePass)
            {
                MRMD_TRY(int32_rows());
                MRMD_TRY(tile_build_launch(ctx, tiles, rows, nPos, nearList, farList, maxCount));
            }
            else if (tiles)
                MRMD_TRY(tile_list_launch(ctx, tiles, rows, nPos, *cl, rsq, rsqLo, rsqHi, nearSqF, nearList,
                                          farList, pos4, maxCount));
            else
                MRMD_TRY(int32_rows());
        }
        int32_t hMax[6] = {0, 0, 0, 0, 0, 0};
        MRMD_CUDA(ctx, cudaMemcpyAsync(hMax, maxCount, 6 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        MRMD_TRY(bounds_check(ctx));
        if (hMax[2]) return set_error(ctx, MRMD_ERR_NONFINITE, "non-finite particle position at the list build");
        if (tiles) tiles->unfitTiles = 0;
        if (tiles && rows > 0 && hMax[4] != 0 && hMax[0] <= capN && hMax[1] <= capF)
        {
            // a tile did not fit the one-pass build: the int32 rows, then
            // their tile form
            tiles->unfitTiles = hMax[4];
            tiles->twoPassBuilds++;
            MRMD_CUDA(ctx, cudaMemsetAsync(maxCount + 3, 0, 3 * sizeof(int32_t), ctx->stream));
            MRMD_TRY(int32_rows());
            MRMD_TRY(tile_build_launch(ctx, tiles, rows, nPos, nearList, farList, maxCount));
            MRMD_CUDA(ctx, cudaMemcpyAsync(hMax, maxCount, 6 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
            MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            MRMD_TRY(bounds_check(ctx));
        }
        if (hMax[0] <= capN && hMax[1] <= capF)
        {
            nearList->rows = farList->rows = rows;
            nearList->begin = farList->begin = begin;
            if (tiles) tile_build_done(tiles, hMax[3], hMax[4] == 0, hMax[5]);
            return MRMD_OK;
        }
        if (hMax[0] > capN) capN = hMax[0] + hMax[0] / 8 + 4;
        if (hMax[1] > capF) capF = hMax[1] + hMax[1] / 8 + 4;
    }
    return set_error(ctx, MRMD_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
}

int list_total_pairs(mrmd_ctx* ctx, mrmd_nlist* nl)
{
    unsigned long long* d = reinterpret_cast<unsigned long long*>(ctx->devScalars + 8);
    MRMD_CUDA(ctx, cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
    if (nl->rows > 0)
    {
        k_count_sum<<<grid_for(ctx, nl->rows, 256, 4), 256, 0, ctx->stream>>>(nl->counts, nl->rows, d);
        MRMD_TRY(after_launch(ctx, "count_sum"));
    }
    unsigned long long h = 0;
    MRMD_CUDA(ctx, cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    nl->totalPairs = (int64_t)h;
    return MRMD_OK;
}

int check_list_fits(mrmd_ctx* ctx, const mrmd_nlist* nl, int64_t numLocal, int64_t nAll)
{
    if (nl->begin < 0 || nl->rows < 0 || nl->begin + nl->rows > numLocal)
        return set_error(ctx, MRMD_ERR_ARG, "list rows [%lld, %lld) exceed the %lld local particles",
                         (long long)nl->begin, (long long)(nl->begin + nl->rows), (long long)numLocal);
    const CellList* cl = static_cast<const CellList*>(nl->cells);
    if (nl->rows > 0 && cl && cl->numParticles > nAll)
        return set_error(ctx, MRMD_ERR_ARG,
                         "list was built over %lld particles but only %lld (local + ghost) are present",
                         (long long)cl->numParticles, (long long)nAll);
    return MRMD_OK;
}

// ----------------------------------------------------------- permutation --

template <typename T>
__global__ void k_gather(const T* __restrict__ src, T* __restrict__ dst, const int32_t* __restrict__ perm,
                         int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

__global__ void k_perm_out(const int32_t* __restrict__ perm, int64_t n, int64_t* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = perm[i];
}

int permute_atoms(mrmd_ctx* ctx, mrmd_atoms* a, mrmd_atoms* shadow, const int32_t* perm, int64_t n)
{
    // gather every field through perm into `shadow`, then swap storage
    constexpr int TB = 256;
    const unsigned gr = grid_for(ctx, n, TB);
    k_gather<double4><<<gr, TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(a->pos),
                                                  reinterpret_cast<double4*>(shadow->pos), perm, n);
    k_gather<double4><<<gr, TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(a->vel),
                                                  reinterpret_cast<double4*>(shadow->vel), perm, n);
    k_gather<double4><<<gr, TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(a->force),
                                                  reinterpret_cast<double4*>(shadow->force), perm, n);
    k_gather<int32_t><<<gr, TB, 0, ctx->stream>>>(a->type, shadow->type, perm, n);
    k_gather<double><<<gr, TB, 0, ctx->stream>>>(a->mass, shadow->mass, perm, n);
    k_gather<double><<<gr, TB, 0, ctx->stream>>>(a->charge, shadow->charge, perm, n);
    k_gather<double><<<gr, TB, 0, ctx->stream>>>(a->relativeMass, shadow->relativeMass, perm, n);
    ctx->launches += 6;
    MRMD_TRY(after_launch(ctx, "permute_gather"));
    std::swap(a->pos, shadow->pos);
    std::swap(a->vel, shadow->vel);
    std::swap(a->force, shadow->force);
    std::swap(a->type, shadow->type);
    std::swap(a->mass, shadow->mass);
    std::swap(a->charge, shadow->charge);
    std::swap(a->relativeMass, shadow->relativeMass);
    return MRMD_OK;
}
}  // namespace mrmd_impl

extern "C" {

int mrmd_nlist_init(mrmd_ctx* ctx, mrmd_nlist* nl)
{
    if (!ctx || !nl) return MRMD_ERR_ARG;
    std::memset(nl, 0, sizeof(*nl));
    nl->cells = new CellList();
    return MRMD_OK;
}

int mrmd_nlist_free(mrmd_ctx* ctx, mrmd_nlist* nl)
{
    if (!nl) return MRMD_ERR_ARG;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(nl->counts);
    dfree(nl->nbrs);
    if (nl->cells)
    {
        CellList* cl = static_cast<CellList*>(nl->cells);
        cl->release();
        delete cl;
    }
    std::memset(nl, 0, sizeof(*nl));
    return MRMD_OK;
}

int mrmd_nlist_build(mrmd_ctx* ctx, mrmd_nlist* nl, const double* pos4, int64_t nPos, int64_t begin,
                     int64_t end, double rlist, double cellRatio, const double* gridMin,
                     const double* gridMax, int64_t maxNeighbors)
{
    if (!ctx || !nl || !nl->cells || !gridMin || !gridMax) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(nPos >= 0 && begin >= 0 && begin <= end && end <= nPos, ctx, "bad particle range");
    MRMD_CHECK_ARG(rlist > 0.0 && cellRatio > 0.0 && cellRatio <= 1.0, ctx, "bad cutoff or cell ratio");
    if (nPos > 0) MRMD_CHECK_ARG(pos4 != nullptr, ctx, "null positions");
    for (int d = 0; d < 3; ++d) MRMD_CHECK_ARG(gridMax[d] > gridMin[d], ctx, "empty grid");
    // cells of edge >= rlist (cellRatio < 1 is accepted and rounded up to one
    // list radius per cell, which keeps the 3-cell stencil exact)
    CellGrid g = make_grid(gridMin, gridMax, rlist);
    (void)cellRatio;
    MRMD_TRY(build_half_list(ctx, nl, pos4, nPos, begin, end, rlist, g, maxNeighbors, false));
    MRMD_TRY(list_total_pairs(ctx, nl));
    return finish(ctx, "nlist_build");
}

int mrmd_nlist_download(mrmd_ctx* ctx, const mrmd_nlist* nl, int32_t* counts, int32_t* nbrs, int64_t cap)
{
    if (!ctx || !nl) return MRMD_ERR_ARG;
    const int64_t rows = nl->rows;
    if (rows == 0) return MRMD_OK;
    std::vector<int32_t> c((size_t)rows);
    MRMD_CUDA(ctx, cudaMemcpyAsync(c.data(), nl->counts, sizeof(int32_t) * (size_t)rows,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int32_t mx = 0;
    for (auto v : c) mx = v > mx ? v : mx;
    if (counts) std::memcpy(counts, c.data(), sizeof(int32_t) * (size_t)rows);
    if (!nbrs) return MRMD_OK;
    if (mx > cap) return set_error(ctx, MRMD_ERR_CAPACITY, "download capacity %lld < %d", (long long)cap, mx);
    const int64_t tiles = div_up(rows, 32), lcap = nl->maxNeighbors;
    std::vector<int32_t> t((size_t)(tiles * 32 * lcap));
    if (mx > 0)
    {
        MRMD_CUDA(ctx, cudaMemcpyAsync(t.data(), nl->nbrs, sizeof(int32_t) * t.size(), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t k = 0; k < c[(size_t)i]; ++k) nbrs[i * cap + k] = t[(size_t)((i >> 5) * (lcap << 5) + (k << 5) + (i & 31))];
    return MRMD_OK;
}

int mrmd_cell_index(mrmd_ctx* ctx, const double* pos4, int64_t n, const double* gridMin,
                    const double* gridMax, double delta, int64_t* cells_out)
{
    if (!ctx || !gridMin || !gridMax || !cells_out || delta <= 0) return MRMD_ERR_ARG;
    if (n == 0) return MRMD_OK;
    CellGrid g = make_grid(gridMin, gridMax, delta);
    CellList cl;
    int rc = cl.build(ctx, pos4, n, g);
    std::vector<int32_t> c((size_t)n);
    if (rc == MRMD_OK)
        rc = check_cuda(ctx, cudaMemcpyAsync(c.data(), cl.cellOf, sizeof(int32_t) * (size_t)n,
                                             cudaMemcpyDeviceToHost, ctx->stream), "cells");
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "cells");
    cl.release();
    if (rc != MRMD_OK) return rc;
    for (int64_t i = 0; i < n; ++i) cells_out[i] = c[(size_t)i];
    return MRMD_OK;
}

int mrmd_atoms_sort_by_cell(mrmd_ctx* ctx, mrmd_atoms* a, const double* gridMin, const double* gridMax,
                            double delta, int64_t* perm_out)
{
    if (!ctx || !a || !gridMin || !gridMax || delta <= 0) return MRMD_ERR_ARG;
    const int64_t n = a->numLocal;
    if (n == 0) return MRMD_OK;
    CellGrid g = make_grid(gridMin, gridMax, delta);
    CellList cl;
    int rc = cl.build(ctx, a->pos, n, g);
    mrmd_atoms shadow{};
    if (rc == MRMD_OK) rc = mrmd_atoms_alloc(ctx, &shadow, a->capacity);
    if (rc == MRMD_OK)
    {
        // ghosts (if any) keep their slots: copy the tail unchanged
        const int64_t tail = a->numGhost;
        if (tail > 0)
        {
            cudaMemcpyAsync(shadow.pos + 4 * n, a->pos + 4 * n, sizeof(double) * 4 * tail, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(shadow.vel + 4 * n, a->vel + 4 * n, sizeof(double) * 4 * tail, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(shadow.force + 4 * n, a->force + 4 * n, sizeof(double) * 4 * tail, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(shadow.type + n, a->type + n, sizeof(int32_t) * tail, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(shadow.mass + n, a->mass + n, sizeof(double) * tail, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(shadow.charge + n, a->charge + n, sizeof(double) * tail, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(shadow.relativeMass + n, a->relativeMass + n, sizeof(double) * tail, cudaMemcpyDeviceToDevice, ctx->stream);
        }
        rc = permute_atoms(ctx, a, &shadow, cl.sorted, n);
    }
    if (rc == MRMD_OK && perm_out)
    {
        int64_t* d = nullptr;
        rc = dmalloc(ctx, reinterpret_cast<void**>(&d), sizeof(int64_t) * (size_t)n);
        if (rc == MRMD_OK)
        {
            k_perm_out<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(cl.sorted, n, d);
            rc = after_launch(ctx, "perm_out");
            if (rc == MRMD_OK)
                rc = check_cuda(ctx, cudaMemcpyAsync(perm_out, d, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream), "perm");
            cudaStreamSynchronize(ctx->stream);
            dfree(d);
        }
    }
    cudaStreamSynchronize(ctx->stream);
    mrmd_atoms_free(ctx, &shadow);  // frees the old storage after the swap
    cl.release();
    return rc;
}

}  // extern "C"
