// The tile form of the near/far split full list (lj_tile.cuh) built in one
// pass from the cell list, without the int32 rows.
//
// One block per tile of TILE_ROWS rows, one thread per row.
// - Span table.  One entry per column (ax, ay) of the stencils of the tile's
//   cells and z block (16 cells) of the asking cell, with the hull of the z
//   ranges those cells ask of the column, in a shared hash table.  An entry's
//   hull (at most 20 cells) is one contiguous span of the cell-sorted
//   particles; numbering the spans one after another gives every candidate
//   of the tile a position (slot = s + delta of its entry).  The z blocks keep
//   two far-apart parts of a tile (a tile across a high Z-order boundary) in
//   separate entries; a particle in the overlap of two entries of a column
//   can become two members, each row using the one of its own entry.
// - Scan.  Each row walks its stencil (for_each_span) with the list builds'
//   exact FP64 pair decision; a kept neighbour marks its candidate position as
//   used and is appended to the row's near or far chunks as that position
//   (16 bits, eight to a chunk, packed in registers).
// - Members.  The used positions are numbered in order (block scan): the
//   tile's members.  Each row then rewrites its own chunks, position ->
//   member slot.
// Rows and the order of a row's entries are those of k_build_list<1, 1>, so
// the pair kernel sums every row in the same order in the tile and the
// gather forms.  A tile whose entries or candidates exceed the tables (rows
// far apart in space: atoms not sorted along the cells) is reported in
// flags[4]; the caller then builds the int32 rows and their tile form.
#include <climits>

#include "common.cuh"
#include "lj_tile.cuh"
#include "nlist_impl.cuh"

using namespace mrmd_impl;

namespace
{
constexpr int COL_BITS = 9;
constexpr int COL_HT = 1 << COL_BITS;  // span table slots per tile (a sorted tile uses ~100-200)
constexpr int ZB_BITS = 4;             // z blocks of 16 cells
constexpr int CAND_CAP = 8192;         // candidate positions per tile (a sorted tile has ~2,000-3,500)

__device__ __forceinline__ uint32_t col_hash(int32_t key)
{
    return ((uint32_t)key * 2654435761u) >> (32 - COL_BITS);
}

// Slot of column `key`, inserted when absent; -1 when the table is full.
__device__ __forceinline__ int col_insert(int32_t* keys, int32_t key)
{
    uint32_t h = col_hash(key);
    for (int probe = 0; probe < COL_HT; ++probe)
    {
        const int32_t k = keys[h];
        if (k == key) return (int)h;
        if (k == -1)
        {
            const int32_t old = atomicCAS(&keys[h], -1, key);
            if (old == -1 || old == key) return (int)h;
        }
        h = (h + 1) & (COL_HT - 1);
    }
    return -1;
}

__device__ __forceinline__ int col_find(const int32_t* keys, int32_t key)
{
    uint32_t h = col_hash(key);
    for (int probe = 0; probe < COL_HT; ++probe)
    {
        const int32_t k = keys[h];
        if (k == key) return (int)h;
        if (k == -1) return -1;
        h = (h + 1) & (COL_HT - 1);
    }
    return -1;
}

// Exclusive prefix of v over the block (TILE_ROWS threads); *total: the sum.
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* warpTot, int32_t* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t incl = v;
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
    *total = warpTot[TILE_ROWS / 32 - 1];
    const int32_t base = (warp > 0 ? warpTot[warp - 1] : 0) + incl - v;
    __syncthreads();  // warpTot is reused by the next scan
    return base;
}

// A row's entries, eight 16-bit values to a 16-byte chunk, shifted in from
// the top so that entry k of a full chunk sits in bits 16 (k % 8).
struct ChunkAcc
{
    uint64_t lo = 0, hi = 0;
    int32_t cnt = 0;
};

__device__ __forceinline__ void chunk_store(uint4* __restrict__ out, int64_t row, int64_t g, int64_t chunks,
                                            uint64_t lo, uint64_t hi)
{
    if (g < chunks)
        out[chunk_word(row, g, chunks)] = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi,
                                                     (uint32_t)(hi >> 32));
}

__device__ __forceinline__ void chunk_push(ChunkAcc& a, uint32_t v, uint4* __restrict__ out, int64_t row,
                                           int64_t chunks)
{
    a.lo = (a.lo >> 16) | (a.hi << 48);
    a.hi = (a.hi >> 16) | ((uint64_t)v << 48);
    ++a.cnt;
    if ((a.cnt & 7) == 0) chunk_store(out, row, (a.cnt >> 3) - 1, chunks, a.lo, a.hi);
}

// The last, partial chunk (entries moved down to bit 0, zeros above).
__device__ __forceinline__ void chunk_flush(const ChunkAcc& a, uint4* __restrict__ out, int64_t row, int64_t chunks)
{
    const int r = a.cnt & 7;
    if (r == 0) return;
    const int k = (8 - r) * 16;  // 16..112
    uint64_t lo, hi;
    if (k >= 64)
    {
        lo = a.hi >> (k - 64);
        hi = 0;
    }
    else
    {
        lo = (a.lo >> k) | (a.hi << (64 - k));
        hi = a.hi >> k;
    }
    chunk_store(out, row, a.cnt >> 3, chunks, lo, hi);
}

// Entries [0, cnt) of a row: candidate positions -> member slots (map).
__device__ __forceinline__ void chunk_remap(uint4* __restrict__ out, int64_t row, int64_t chunks, int32_t cnt,
                                            const int32_t* map, int32_t nMap)
{
    for (int32_t g0 = 0; g0 < cnt; g0 += 8)
    {
        const int64_t w = chunk_word(row, g0 >> 3, chunks);
        const uint4 c = out[w];  // written by this thread above
        uint32_t v[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
        {
            const int32_t e = g0 + 2 * q;
            const int32_t p0 = (int32_t)(v[q] & 0xffffu), p1 = (int32_t)(v[q] >> 16);
            const uint32_t m0 = e < cnt && p0 < nMap ? (uint32_t)map[p0] & 0xffffu : 0u;
            const uint32_t m1 = e + 1 < cnt && p1 < nMap ? (uint32_t)map[p1] & 0xffffu : 0u;
            v[q] = m0 | (m1 << 16);
        }
        out[w] = make_uint4(v[0], v[1], v[2], v[3]);
    }
}

// flags: [0], [1] longest near / far row, [3] largest member count, [4] tiles
// that did not fit (their rows are incomplete), [5] members of all tiles.
// Four blocks per SM (64 registers): the scan is bound by the latency of its
// candidate loads; three blocks of 72 registers ran 14% slower.
__global__ void __launch_bounds__(TILE_ROWS, 4) k_tile_list(
    const double4* __restrict__ pos, const int32_t* __restrict__ cellOf, const int32_t* __restrict__ cellStart,
    const float4* __restrict__ spos, CellGrid g, int64_t rows, int64_t nPos, double rsq,
    float rsqLo, float rsqHi, float nearSqF, int64_t capN, int64_t capF, int32_t* __restrict__ countsN,
    int32_t* __restrict__ countsF, int32_t* __restrict__ flags, int32_t* __restrict__ members,
    int32_t* __restrict__ memberCount, uint4* __restrict__ nearChunks, int64_t chN, uint4* __restrict__ farChunks,
    int64_t chF)
{
    __shared__ int32_t colKey[COL_HT], colLo[COL_HT], colHi[COL_HT], colDelta[COL_HT];
    __shared__ int32_t used[CAND_CAP];  // candidate position -> particle (-1: unused), then -> member slot
    __shared__ int32_t warpTot[TILE_ROWS / 32];
    __shared__ int32_t badS;
    const int tid = threadIdx.x, lane = tid & 31;
    const int64_t tile = blockIdx.x;
    const int64_t row = tile * TILE_ROWS + tid;
    for (int h = tid; h < COL_HT; h += TILE_ROWS)
    {
        colKey[h] = -1;
        colLo[h] = INT_MAX;
        colHi[h] = -1;
    }
    if (tid == 0) badS = 0;
    __syncthreads();

    // ---- span table: one insertion per distinct cell of a warp's rows
    const int nzb = ((g.n.z - 1) >> ZB_BITS) + 1;
    bool live = row < rows;
    int32_t ci = live ? cellOf[row] : -1;
    if (live && !MRMD_IN_BOUNDS(ci, g.ncell)) live = false;
    const int32_t prev = __shfl_up_sync(0xffffffffu, ci, 1);
    if (live && (lane == 0 || prev != ci))
    {
        const int cz = ci % g.n.z, cy = (ci / g.n.z) % g.n.y, cx = ci / (g.n.z * g.n.y);
        const int R = g.reach;
        const int z0 = max(cz - R, 0), z1 = min(cz + R, g.n.z - 1);
        for (int ax = max(cx - R, 0); ax <= min(cx + R, g.n.x - 1); ++ax)
            for (int ay = max(cy - R, 0); ay <= min(cy + R, g.n.y - 1); ++ay)
            {
                const int h = col_insert(colKey, (ax * g.n.y + ay) * nzb + (cz >> ZB_BITS));
                if (h < 0)
                {
                    badS = 1;
                    continue;
                }
                atomicMin(&colLo[h], z0);
                atomicMax(&colHi[h], z1);
            }
    }
    __syncthreads();

    // ---- candidate positions: the entries' spans numbered one after another
    constexpr int PER = COL_HT / TILE_ROWS;
    int32_t cnt[PER], start[PER];
    int32_t local = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q)
    {
        const int h = tid * PER + q;
        const int32_t key = colKey[h];
        cnt[q] = 0;
        start[q] = 0;
        if (key >= 0)
        {
            const int64_t c0 = (int64_t)(key / nzb) * g.n.z;
            const int64_t a = c0 + colLo[h], b = c0 + colHi[h] + 1;
            if (MRMD_IN_BOUNDS(a, g.ncell) && MRMD_IN_BOUNDS(b, g.ncell + 1))
            {
                start[q] = cellStart[a];
                cnt[q] = cellStart[b] - start[q];
            }
        }
        local += cnt[q];
    }
    int32_t nCand;
    int32_t base = block_exclusive_scan(local, warpTot, &nCand);
#pragma unroll
    for (int q = 0; q < PER; ++q)
    {
        colDelta[tid * PER + q] = base - start[q];
        base += cnt[q];
    }
    for (int32_t p = tid; p < nCand && p < CAND_CAP; p += TILE_ROWS) used[p] = -1;
    __syncthreads();
    if (badS || nCand > CAND_CAP)
    {
        if (tid == 0) atomicAdd(&flags[4], 1);
        return;
    }

    // ---- scan: the rows' neighbours as candidate positions
    ChunkAcc an, af;
    if (live)
    {
        const double4 pi = pos[row];
        const float xi = (float)(pi.x - g.mn.x), yi = (float)(pi.y - g.mn.y), zi = (float)(pi.z - g.mn.z);
        auto candidate = [&](const float4& q, int32_t slot) {
            float d2f;
            if (!candidate_kept<true>(pos, pi, row, xi, yi, zi, q, rsq, rsqLo, rsqHi, nPos, d2f)) return;
            if ((uint32_t)slot >= (uint32_t)nCand) return;  // unreachable: the span lies in its entry's hull
            used[slot] = __float_as_int(q.w);
            if (d2f >= nearSqF)
                chunk_push(af, (uint32_t)slot, farChunks, row, chF);
            else
                chunk_push(an, (uint32_t)slot, nearChunks, row, chN);
        };
        const int zbRow = (ci % g.n.z) >> ZB_BITS;
        for_each_span<true>(cellStart, g, ci, nPos, [&](int ax, int ay, int32_t, int, int, int32_t s0, int32_t s1) {
            const int h = col_find(colKey, (ax * g.n.y + ay) * nzb + zbRow);
            if (h < 0) return;  // unreachable: the table holds every entry of the row's stencil
            const int32_t delta = colDelta[h];
            int32_t s = s0;
            for (; s + 3 < s1; s += 4)
            {
                const float4 q0 = spos[s], q1 = spos[s + 1], q2 = spos[s + 2], q3 = spos[s + 3];
                candidate(q0, s + delta);
                candidate(q1, s + 1 + delta);
                candidate(q2, s + 2 + delta);
                candidate(q3, s + 3 + delta);
            }
            for (; s < s1; ++s) candidate(spos[s], s + delta);
        });
        chunk_flush(an, nearChunks, row, chN);
        chunk_flush(af, farChunks, row, chF);
        countsN[row] = an.cnt < capN ? an.cnt : (int32_t)capN;
        countsF[row] = af.cnt < capF ? af.cnt : (int32_t)capF;
        if (an.cnt > capN) atomicMax(&flags[0], an.cnt);
        if (af.cnt > capF) atomicMax(&flags[1], af.cnt);
    }
    __syncthreads();

    // ---- members: the used positions in order
    const int32_t per = (nCand + TILE_ROWS - 1) / TILE_ROWS;
    const int32_t p0 = tid * per, p1 = min(p0 + per, nCand);
    local = 0;
    for (int32_t p = p0; p < p1; ++p) local += used[p] >= 0;
    int32_t total;
    int32_t m = block_exclusive_scan(local, warpTot, &total);
    int32_t* mem = members + tile * TILE_CAP;
    for (int32_t p = p0; p < p1; ++p)
    {
        const int32_t j = used[p];
        if (j < 0) continue;
        if (m < TILE_CAP) mem[m] = j;
        used[p] = m++;
    }
    if (tid == 0)
    {
        memberCount[tile] = total < TILE_CAP ? total : TILE_CAP;
        atomicMax(&flags[3], total);
        atomicAdd(&flags[5], total);
        if (total > TILE_CAP) atomicAdd(&flags[4], 1);
    }
    __syncthreads();
    if (total > TILE_CAP || !live) return;

    // ---- each row's entries: candidate positions -> member slots
    chunk_remap(nearChunks, row, chN, an.cnt < capN ? an.cnt : (int32_t)capN, used, nCand);
    chunk_remap(farChunks, row, chF, af.cnt < capF ? af.cnt : (int32_t)capF, used, nCand);
}
}  // namespace

namespace mrmd_impl
{
int tile_list_launch(mrmd_ctx* ctx, TileList* tl, int64_t rows, int64_t nPos, const CellList& cl, double rsq,
                     float rsqLo, float rsqHi, float nearSqF, mrmd_nlist* nearList, mrmd_nlist* farList,
                     const double* pos4, int32_t* flags)
{
    MRMD_TRY(tile_storage(ctx, tl, rows, nearList->maxNeighbors, farList->maxNeighbors));
    if (rows == 0) return MRMD_OK;
    k_tile_list<<<(unsigned)tl->tiles, TILE_ROWS, 0, ctx->stream>>>(
        reinterpret_cast<const double4*>(pos4), cl.cellOf, cl.cellStart, cl.spos, cl.g, rows, nPos, rsq, rsqLo, rsqHi,
        nearSqF, nearList->maxNeighbors, farList->maxNeighbors, nearList->counts, farList->counts, flags, tl->members,
        tl->memberCount, tl->nearChunks, tl->nearChunksPerRow, tl->farChunks, tl->farChunksPerRow);
    return after_launch(ctx, "tile_list");
}
}  // namespace mrmd_impl
