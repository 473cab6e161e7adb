// Mixed-form LJ pair force of the fused stepper: neighbour records staged in
// shared-memory tiles, r^2 exact as a float pair, far pairs in FP32.
//
// Coordinates.  c = x - origin (origin = the cell grid's corner) is split into
//   hi = c rounded to a multiple of Q = 2^-q, with 2^11 Q > r_list, and
//   lo = float(c - hi), |lo| <= Q / 2.
// For a pair within the list radius, dh = hi_i - hi_j is an exact FP32 value
// k Q with |k| < 2^11, so dh^2 (k^2 Q^2, k^2 < 2^22) and the sum of the three
// squares (< 3 * 2^22 quanta of Q^2) are exact in FP32.  With dl = lo_i - lo_j,
// r^2 = S + C where S = sum dh^2 (exact) and C = sum dl (2 dh + dl) (small,
// FP32-accurate): r^2 is known as the float pair (S + C, rounding error) to
// about 2^-44 relative.
//
// Records.  Per particle A = (hi.x, hi.y, hi.z, lo.x) and B = (lo.y, lo.z):
// 24 bytes.  The stepper writes them in its kick/drift and ghost-update
// kernels; the pair kernel copies the records of a tile's neighbours into
// shared memory once per step.
//
// Tiles.  TILE_ROWS consecutive list rows (atoms, cell-sorted) form a tile.
// Its members are the distinct neighbours of its rows; the rows store
// 16-bit member slots instead of particle indices, eight to a 16-byte chunk.
#pragma once

#include <cstdint>

#include "lj_impl.cuh"
#include "lj_mixed.cuh"

namespace mrmd_impl
{
constexpr int TILE_ROWS = 256;
// members per tile the build's shared hash table allows (a 256-row tile of
// the dense LJ fluid, rho 0.8442 and r_list 2.8 sigma, has about 1,400-2,200)
constexpr int TILE_CAP = 3072;

// Split parameters with the quantum Q = 2^-q of the tile kernel for list
// radius rlist: the largest Q with 2^11 Q > rlist * 1.0625, and `origin`
// rounded down to a multiple of Q.  Coordinates relative to the origin must
// stay below 2^24 Q in magnitude (`extent` bounds them); returns false
// otherwise.
bool tile_split_params(const double* origin, double extent, double rlist, SplitParams* out);

// (A, B) records of one position: the split of each coordinate relative to
// the origin (a multiple of Q) on the integer pipe (split_bits: the same bits
// as rounding x + (magic - origin) to the Q grid in FP64; no FP64 operation).
__device__ __forceinline__ void tile_split(const double4& x, const SplitParams& sp, float4& a, float2& b)
{
    float lx, ly, lz;
    split_bits(x.x, sp.ko.x, sp.q, sp.invScaleF, a.x, lx);
    split_bits(x.y, sp.ko.y, sp.q, sp.invScaleF, a.y, ly);
    split_bits(x.z, sp.ko.z, sp.q, sp.invScaleF, a.z, lz);
    a.w = lx;
    b = make_float2(ly, lz);
}

// Records of particles [0, n) into recA / recB.
int tile_split_coords(mrmd_ctx* ctx, const double* pos4, int64_t n, const SplitParams& sp, float4* recA,
                      float2* recB);

// Rows of member slots in 8-entry chunks: chunk g of row i is the 16-byte
// word (i / 32) * chunks * 32 + 32 g + i % 32 (chunks = ceil(capacity / 8)),
// and entry k of the row is 16-bit lane k % 8 of chunk k / 8.  A warp reads
// chunk g of its 32 rows as 512 contiguous bytes, eight pairs per lane.
__host__ __device__ inline int64_t chunk_word(int64_t row, int64_t g, int64_t chunks)
{
    return (row >> 5) * (chunks << 5) + (g << 5) + (row & 31);
}

// The tile form of a near/far split full list (build_split_list).  Rows and
// counts follow the two int32 lists; entries are member slots.
struct TileList
{
    int32_t* members = nullptr;      // [tiles][TILE_CAP] particle index of each member
    int32_t* memberCount = nullptr;  // [tiles]
    uint4* nearChunks = nullptr;     // near rows
    uint4* farChunks = nullptr;      // far rows
    int64_t nearChunksPerRow = 0, farChunksPerRow = 0;
    int64_t tilesCap = 0, nearWords = 0, farWords = 0;  // allocated
    int64_t tiles = 0;
    int32_t maxMembers = 0;  // largest tile after the last build
    int64_t totalMembers = 0;  // members of all tiles after the last build
    bool valid = false;      // every tile fits TILE_CAP
    int64_t unfitTiles = 0;     // tiles the last one-pass build could not fit
    int64_t twoPassBuilds = 0;  // builds that made the int32 rows and their tile form
    void release();
};

// Storage of tl for `rows` rows with near / far row capacities capN / capF
// (entries); also raises the pair kernel's shared-memory limit.
int tile_storage(mrmd_ctx* ctx, TileList* tl, int64_t rows, int64_t capN, int64_t capF);

// The tile form of a near/far split full list over rows [0, rows) of
// particles [0, nAll), from its int32 rows, launched right after the list
// build (one block per tile: the distinct neighbours of its rows get slots
// through a shared-memory hash table); flags: the build's device flags (see
// k_tile_build).  The one-pass build (tile_list_launch, nlist_impl.cuh) makes
// the same form from the cell list.  tile_build_done records what the caller
// read back; tl->valid is false when a tile has more than TILE_CAP members.
int tile_build_launch(mrmd_ctx* ctx, TileList* tl, int64_t rows, int64_t nAll, const mrmd_nlist* nearList,
                      const mrmd_nlist* farList, int32_t* flags);
void tile_build_done(TileList* tl, int32_t maxMembers, bool valid, int64_t totalMembers);

// Per-system constants of the pair kernel.
struct TileParams
{
    LJDev p;
    RcSq rc2;
    float rsplitSq;
    float bias3, bias6;  // offsets of the u^3, u^6 sums (make_tile_params)
};

TileParams make_tile_params(const LJDev& p, double rcSqr, double rsplit, int64_t farCapacity);

// Forces of local atoms [0, rows) written into force4 (overwritten, ghosts
// untouched), energy and virial added into ev[0], ev[1].  With a valid tile
// list the neighbour records come from shared-memory tiles; otherwise (or
// with `gather` set) they are gathered from recA / recB through the int32
// lists.
int lj_tile_forces(mrmd_ctx* ctx, const TileList* tl, const mrmd_nlist* nearList, const mrmd_nlist* farList,
                   const float4* recA, const float2* recB, double* force4, const TileParams& tp, double* ev,
                   int64_t nAll, bool gather);
}  // namespace mrmd_impl
