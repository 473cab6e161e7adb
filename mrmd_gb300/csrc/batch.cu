// Batched AdResS replicas: many independent single-site LJ <-> ideal-gas
// systems of different sizes and geometries advanced together, one kernel
// launch per phase for all replicas, replayed as CUDA graphs.
//
// Each replica follows the step of the fused single-system stepper
// (VelocityVerletLangevinThermostat pre, MultiResGhostLayer, UpdateMolecules
// with a Slab, LJ_IdealGas::run, ContributeMoleculeForceToAtoms,
// ThermodynamicForce apply/sample/update, VelocityVerlet post).  The layout
// and the kernels are designed for one GPU holding all replicas at once:
//
//  * one flat slot space: the local molecules of all replicas, replica after
//    replica, then all ghosts; every slot knows its replica, every replica
//    its box, slab, cell grid, noise key and thermodynamic-force table;
//  * rebuild decisions, ghost counts and list overflow live on the device,
//    so a whole graph of steps (rebuilds included) runs without the host;
//    overflow is detected after the graph, the state restored from a
//    snapshot taken before it and the graph re-run with larger buffers;
//  * the pair force walks a FULL molecule list and writes each local force
//    once: no atomics, no ghost forces, no fold-back, and the result is
//    bitwise independent of the other replicas.  For a pair with a ghost the
//    kernel uses the weights of the pair instance that Cabana's half list
//    (lexicographic order) keeps in the reference, so that boxes whose slab
//    reaches into the ghost layer see the reference's weights exactly;
//  * TF application, the velocity-Verlet post kick, density sampling and
//    the drift-compensation sampling are fused into the pair kernel's
//    epilogue; the per-replica table updates run in one tail kernel with one
//    block per replica.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "adress_impl.cuh"
#include "common.cuh"
#include "integrate_impl.cuh"
#include "lj_impl.cuh"
#include "lj_mixed.cuh"
#include "nlist_impl.cuh"
#include "thermo_impl.cuh"
#include "batch_impl.cuh"

using namespace mrmd_impl;
using namespace mrmd_batch_impl;

namespace
{
// ------------------------------------------------------------------ pre --
// B(dt/2) A(dt/2) O(dt) A(dt/2) (VelocityVerletLangevinThermostat.hpp:64-113)
// with noise keyed by (replica seed, step, the molecule's input index inside
// the replica: the noise follows the molecule through cell sorts); on a
// rebuild step the molecule is then wrapped into its box by the
// MultiResRealAtomsExchange rule (MultiResRealAtomsExchange.cpp:23-73).
// The body over molecules tid, tid + stride, ... (every thread of the grid
// calls it: the displacement maximum ends in a warp reduction).
template <bool MIXED>
__device__ __forceinline__ void pre_body(const BDev& B, int rebuild, int64_t tid, int64_t stride)
{
    const unsigned long long st = B.sc->step;
    for (int64_t r = tid; r < B.R; r += stride) B.energyRing[(int64_t)B.sc->ringSlot * B.R + r] = 0.0;
    float m2 = 0.0f;
    const double dtHalf = 0.5 * B.dt;
    for (int64_t i = tid; i < B.N; i += stride)
    {
        const RepDev& R = B.reps[B.slotRep[i]];
        double4 x = B.pos[i], v = B.vel[i];
        const double4 f = B.force[i];
        const double m = B.mass[i];
        (void)m;  // unit masses: dt/2m and the OU coefficients are constants
        kick_fma(v, f, B.dtHalfOverMass);
        drift_fma(x, v, dtHalf);
        double g[3];
        normal3(R.seed, st, (uint64_t)(B.orig[i] - R.lbase), g);
        v.x = fma(B.ouSigma, g[0], v.x * B.ouDamping);
        v.y = fma(B.ouSigma, g[1], v.y * B.ouDamping);
        v.z = fma(B.ouSigma, g[2], v.z * B.ouDamping);
        drift_fma(x, v, dtHalf);
        // Verlet criterion: displacement since the list was built (FP32; the
        // bound it is compared with, skin/2, is far above the rounding)
        const float4 r0 = B.ref[i];
        if (MIXED && !rebuild)
        {
            // r0 is relative to gmn, the split coordinates to the split
            // origin, soff below it
            B.pos[i] = x;
            B.vel[i] = v;
            float4 h, l;
            slot_derived<MIXED>(B, R, i, x, &h, &l);
            const float dx = ((h.x - r0.x) + l.x) - R.soff[0], dy = ((h.y - r0.y) + l.y) - R.soff[1],
                        dz = ((h.z - r0.z) + l.z) - R.soff[2];
            m2 = fmaxf(m2, __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz))));
            continue;
        }
        {
            const float dx = (float)(x.x - R.gmn[0]) - r0.x, dy = (float)(x.y - R.gmn[1]) - r0.y,
                        dz = (float)(x.z - R.gmn[2]) - r0.z;
            m2 = fmaxf(m2, __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz))));
        }
        if (rebuild)
        {
#pragma unroll
            for (int d = 0; d < 3; ++d)
            {
                double c = coord(x, d);
                if (R.mx[d] <= c) c = __dsub_rn(c, R.L[d]);
                if (c < R.lo[d]) c = __dadd_rn(c, R.L[d]);
                set_coord(x, d, c);
            }
        }
        B.pos[i] = x;
        B.vel[i] = v;
        slot_derived<MIXED>(B, R, i, x);
    }
    for (int o = 16; o > 0; o >>= 1) m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    if ((threadIdx.x & 31) == 0) mrmd_dev::atomic_max_nonneg(&B.sc->dispStep, (double)m2);
}

template <bool MIXED>
__global__ void k_b_pre(BDev B, int rebuild)
{
    pre_body<MIXED>(B, rebuild, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// weights and split coordinates of the locals at their current positions
template <bool MIXED>
__global__ void k_b_derive(BDev B)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B.N; i += (int64_t)gridDim.x * blockDim.x)
        slot_derived<MIXED>(B, B.reps[B.slotRep[i]], i, B.pos[i]);
}

// ----------------------------------------------------------------- cells --
__device__ __forceinline__ int32_t rep_cell(const RepDev& R, const double4& p)
{
    int32_t c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        const double t = floor(__dmul_rn(__dsub_rn(coord(p, d), R.gmn[d]), R.grdx[d]));
        c[d] = t >= 0.0 ? (t > (double)(R.gn[d] - 1) ? R.gn[d] - 1 : (int)t) : 0;  // NaN: cell 0
    }
    return R.cellBase + (c[0] * R.gn[1] + c[1]) * R.gn[2] + c[2];
}

__device__ __forceinline__ int32_t num_slots(const BDev& B, int withGhosts)
{
    if (!withGhosts) return B.N;
    const int32_t g = B.sc->numGhost;
    return B.N + (g < B.gCap ? g : B.gCap);
}

__global__ void k_b_cell_count(BDev B, int withGhosts)
{
    const int32_t n = num_slots(B, withGhosts);
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const int32_t c = rep_cell(B.reps[B.slotRep[s]], B.pos[s]);
        B.cellOf[s] = c;
        atomicAdd(&B.cellStart[c], 1);
    }
}

__global__ void k_b_cell_scatter(BDev B, int withGhosts)
{
    const int32_t n = num_slots(B, withGhosts);
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const int32_t c = B.cellOf[s];
        B.unordered[B.cellStart[c] + atomicAdd(&B.cursor[c], 1)] = s;
    }
}

// stable order inside each cell (ascending slot), then FP32 coordinates
// relative to the replica's grid origin with the slot in w
__global__ void k_b_cell_rank(BDev B, int withGhosts)
{
    const int32_t n = num_slots(B, withGhosts);
    for (int32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    {
        const int32_t v = B.unordered[t];
        const int32_t c = B.cellOf[v];
        const int32_t b = B.cellStart[c], e = B.cellStart[c + 1];
        int32_t rank = 0;
        for (int32_t u = b; u < e; ++u) rank += B.unordered[u] < v;
        B.sorted[b + rank] = v;
        if (withGhosts)
        {
            const RepDev& R = B.reps[B.slotRep[v]];
            const double4 p = B.pos[v];
            B.spos[b + rank] = make_float4((float)(p.x - R.gmn[0]), (float)(p.y - R.gmn[1]),
                                           (float)(p.z - R.gmn[2]), __int_as_float(v));
        }
    }
}

// ----------------------------------------------------------- local sort --
__global__ void k_b_sort_gather(BDev B)
{
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < B.N; s += gridDim.x * blockDim.x)
    {
        const int32_t src = B.sorted[s];
        B.sPos[s] = B.pos[src];
        B.sVel[s] = B.vel[src];
        B.sMass[s] = B.mass[src];
        B.sOrig[s] = B.orig[src];
    }
}

template <bool MIXED>
__global__ void k_b_sort_store(BDev B)
{
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < B.N; s += gridDim.x * blockDim.x)
    {
        const double4 x = B.sPos[s];
        B.pos[s] = x;
        B.vel[s] = B.sVel[s];
        B.mass[s] = B.sMass[s];
        B.orig[s] = B.sOrig[s];
        slot_derived<MIXED>(B, B.reps[B.slotRep[s]], s, x);
    }
}

// --------------------------------------------------------------- ghosts --
// Images of each local molecule: per axis x < minInner gives a +L image and
// x >= maxInner a -L image (MultiResPeriodicGhostExchange.cpp:60-248, ghosts
// of ghosts included), i.e. the product over the axes minus the molecule.
__global__ void k_b_ghost_count(BDev B)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B.N; i += gridDim.x * blockDim.x)
    {
        const RepDev& R = B.reps[B.slotRep[i]];
        const double4 x = B.pos[i];
        uint32_t flags = 0;
        int32_t n = 1;
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            const double c = coord(x, d);
            const bool plus = c < R.minIn[d], minus = c >= R.maxIn[d];
            flags |= (plus ? 1u : 0u) << (2 * d);
            flags |= (minus ? 1u : 0u) << (2 * d + 1);
            n *= 1 + (int)plus + (int)minus;
        }
        B.imgFlags[i] = (uint8_t)flags;
        B.gCount[i] = n - 1;
        B.xImg[i] = make_int2(-1, -1);
        B.ref[i] = make_float4((float)(x.x - R.gmn[0]), (float)(x.y - R.gmn[1]), (float)(x.z - R.gmn[2]), 0.0f);
    }
}

template <bool MIXED>
__global__ void k_b_ghost_write(BDev B)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B.N; i += gridDim.x * blockDim.x)
    {
        const int32_t r = B.slotRep[i];
        const RepDev& R = B.reps[r];
        const uint32_t flags = B.imgFlags[i];
        const double4 x = B.pos[i];
        int32_t k = B.gCount[i];  // exclusive offset
        int2 xImg = make_int2(-1, -1);
        // options per axis: 0 (no shift), 2 (-L) if x >= maxInner, 1 (+L) if x < minInner
        for (int ox = 0; ox < 3; ++ox)
        {
            const int cx = ox == 0 ? 0 : (ox == 1 ? 2 : 1);
            if (cx && !(flags & (cx == 1 ? 1u : 2u))) continue;
            for (int oy = 0; oy < 3; ++oy)
            {
                const int cy = oy == 0 ? 0 : (oy == 1 ? 2 : 1);
                if (cy && !(flags & (cy == 1 ? 4u : 8u))) continue;
                for (int oz = 0; oz < 3; ++oz)
                {
                    const int cz = oz == 0 ? 0 : (oz == 1 ? 2 : 1);
                    if (cz && !(flags & (cz == 1 ? 16u : 32u))) continue;
                    if (!cx && !cy && !cz) continue;
                    const int32_t g = k++;
                    if (g >= B.gCap)
                    {
                        atomicOr(&B.sc->overflow, FLAG_GHOST_OVERFLOW);
                        continue;
                    }
                    double4 p = x;
                    const int c3[3] = {cx, cy, cz};
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                    {
                        if (c3[d] == 1) set_coord(p, d, __dadd_rn(coord(p, d), R.L[d]));
                        if (c3[d] == 2) set_coord(p, d, __dsub_rn(coord(p, d), R.L[d]));
                    }
                    p.w = 0.0;
                    const int64_t s = (int64_t)B.N + g;
                    B.pos[s] = p;
                    B.slotRep[s] = r;
                    B.gSrc[g] = i;
                    B.gShift[g] = (uint8_t)(cx | (cy << 2) | (cz << 4));
                    slot_derived<MIXED>(B, R, s, p);
                    if (!cy && !cz)
                    {
                        if (cx == 2) xImg.x = (int32_t)s;
                        if (cx == 1) xImg.y = (int32_t)s;
                    }
                }
            }
        }
        B.xImg[i] = xImg;
    }
}

// ghost position = real position +- L (UpdateGhostAtoms.cpp:31-68)
template <bool MIXED>
__device__ __forceinline__ void ghost_update_body(const BDev& B, int64_t tid, int64_t stride)
{
    const int32_t n = num_slots(B, 1) - B.N;
    for (int64_t g = tid; g < n; g += stride)
    {
        const int32_t i = B.gSrc[g];
        const uint32_t code = B.gShift[g];
        const RepDev& R = B.reps[B.slotRep[i]];
        double4 p = B.pos[i];
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            const uint32_t c = (code >> (2 * d)) & 3u;
            if (c == 1) set_coord(p, d, __dadd_rn(coord(p, d), R.L[d]));
            if (c == 2) set_coord(p, d, __dsub_rn(coord(p, d), R.L[d]));
        }
        p.w = 0.0;
        const int64_t s = (int64_t)B.N + g;
        B.pos[s] = p;
        slot_derived<MIXED>(B, R, s, p);
    }
}

template <bool MIXED>
__global__ void k_b_ghost_update(BDev B)
{
    ghost_update_body<MIXED>(B, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// ------------------------------------------------------------ list build --
// Cabana's half-list discriminator (lexicographic x, y, z): b above a
__device__ __forceinline__ bool lex_above(const double4& a, const double4& b)
{
    return (b.x > a.x) || ((b.x == a.x) && ((b.y > a.y) || ((b.y == a.y) && (b.z > a.z))));
}

// Full list (every slot j != i of the same replica within r_list) of each
// local molecule, 27-cell stencil walked as contiguous z-column spans of the
// replica's cell-sorted FP32 coordinates; an FP32 prefilter settles the
// clear cases and FP64 positions decide inside its error band.
__global__ void __launch_bounds__(128) k_b_build_list(BDev B)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < B.N; i += gridDim.x * blockDim.x)
    {
        const RepDev& R = B.reps[B.slotRep[i]];
        const double4 pi = B.pos[i];
        const float xi = (float)(pi.x - R.gmn[0]), yi = (float)(pi.y - R.gmn[1]), zi = (float)(pi.z - R.gmn[2]);
        const uint32_t myImg = B.imgFlags[i];
        // molecules that stay coarse grained (ideal gas) until the next rebuild
        // interact with no other such molecule: their pairs are left out
        const float deepCG = (float)(R.slab.atHalf + R.slab.hy + B.cgMargin);
        const float cxRel = (float)(R.slab.cx - R.gmn[0]);
        const bool prune = R.consistent != 0;
        const bool rowCG = prune && fabsf(xi - cxRel) > deepCG;
        const int32_t ci = B.cellOf[i] - R.cellBase;
        const int cz = ci % R.gn[2];
        const int cy = (ci / R.gn[2]) % R.gn[1];
        const int cx = ci / (R.gn[2] * R.gn[1]);
        int32_t cnt = 0, cntF = 0;
        const int az0 = max(cz - 1, 0), az1 = min(cz + 1, R.gn[2] - 1);
        for (int ax = max(cx - 1, 0); ax <= min(cx + 1, R.gn[0] - 1); ++ax)
        {
            for (int ay = max(cy - 1, 0); ay <= min(cy + 1, R.gn[1] - 1); ++ay)
            {
                const int32_t c0 = R.cellBase + (ax * R.gn[1] + ay) * R.gn[2];
                const int32_t s0 = B.cellStart[c0 + az0], s1 = B.cellStart[c0 + az1 + 1];
                for (int32_t s = s0; s < s1; ++s)
                {
                    const float4 q = B.spos[s];
                    const int32_t j = __float_as_int(q.w);
                    if (j == i) continue;
                    if (rowCG && fabsf(q.x - cxRel) > deepCG) continue;
                    const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
                    const float d2f = dx * dx + dy * dy + dz * dz;
                    if (d2f > B.listRsqHi) continue;
                    bool keep = d2f < B.listRsqLo;
                    if (!keep)
                    {
                        const double4 pj = B.pos[j];
                        const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
                        const double d2 =
                            __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
                        keep = d2 <= B.listRsq;
                    }
                    if (!keep) continue;
                    int32_t entry = j;
                    if (j >= B.N && !lex_above(pi, B.pos[j]))
                    {
                        // Cabana's half list keeps (source, image of i) instead of
                        // (i, ghost): i must have that image, or the pair is absent
                        const uint32_t code = B.gShift[j - B.N];
                        bool has = true;
#pragma unroll
                        for (int d = 0; d < 3; ++d)
                        {
                            const uint32_t c = (code >> (2 * d)) & 3u;
                            if (c == 1) has = has && (myImg & (2u << (2 * d)));  // ghost +L: i needs a -L image
                            if (c == 2) has = has && (myImg & (1u << (2 * d)));  // ghost -L: i needs a +L image
                        }
                        if (!has) continue;
                        entry = j | REVERSED;
                    }
                    if (B.split && d2f >= B.nearSqF)
                    {
                        if (cntF < B.listCapF) B.nbrsF[mrmd_dev::nbr_row(i, B.listCapF) + 32 * (int64_t)cntF] = entry;
                        ++cntF;
                        continue;
                    }
                    if (cnt < B.listCap) B.nbrs[mrmd_dev::nbr_row(i, B.listCap) + 32 * (int64_t)cnt] = entry;
                    ++cnt;
                }
            }
        }
        B.counts[i] = cnt < B.listCap ? cnt : B.listCap;
        if (cnt > B.listCap)
        {
            atomicMax(&B.sc->maxCount, cnt);
            atomicOr(&B.sc->overflow, FLAG_LIST_OVERFLOW);
        }
        if (B.split)
        {
            B.countsF[i] = cntF < B.listCapF ? cntF : B.listCapF;
            if (cntF > B.listCapF)
            {
                atomicMax(&B.sc->maxCountF, cntF);
                atomicOr(&B.sc->overflow, FLAG_FAR_LIST_OVERFLOW);
            }
        }
    }
}

// Cluster-pair list (8 x 4 layout) of each i-cluster, one warp per cluster:
// the warp walks the union of its rows' 27-cell stencils as z-column spans of
// the replica's cell-sorted slots, in j-clusters of CLUSTER_J slots aligned to
// the replica's first sorted position.  Lane 4a + b tests row a against slot
// b of the j-cluster with the tests of k_b_build_list (same pairs, same
// reversed instances); a cluster pair with any pair kept is stored with the
// ballots of the kept and the reversed pairs.  Spans come in ascending sorted
// order, so a j-cluster shared by two spans is visited once.
__global__ void __launch_bounds__(128) k_b_build_clusters(BDev B)
{
    const int lane = threadIdx.x & 31;
    const int a = lane >> 2, sb = lane & (CLUSTER_J - 1);
    const int32_t nw = (int32_t)((gridDim.x * blockDim.x) >> 5);
    for (int32_t c = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < B.numClusters; c += nw)
    {
        const int2 cl = B.clusters[c];
        const bool rowValid = a < cl.y;
        const int32_t i = cl.x + (rowValid ? a : 0);  // rows past the cluster's end repeat row 0
        const RepDev& R = B.reps[B.slotRep[cl.x]];
        const double4 pi = B.pos[i];
        const float xi = (float)(pi.x - R.gmn[0]), yi = (float)(pi.y - R.gmn[1]), zi = (float)(pi.z - R.gmn[2]);
        const uint32_t myImg = B.imgFlags[i];
        const float deepCG = (float)(R.slab.atHalf + R.slab.hy + B.cgMargin);
        const float cxRel = (float)(R.slab.cx - R.gmn[0]);
        const bool rowCG = R.consistent != 0 && fabsf(xi - cxRel) > deepCG;
        const int32_t ci = B.cellOf[i] - R.cellBase;
        const int cz = ci % R.gn[2];
        const int cy = (ci / R.gn[2]) % R.gn[1];
        const int cx = ci / (R.gn[2] * R.gn[1]);
        const int x0 = __reduce_min_sync(0xffffffffu, cx), x1 = __reduce_max_sync(0xffffffffu, cx);
        const int y0 = __reduce_min_sync(0xffffffffu, cy), y1 = __reduce_max_sync(0xffffffffu, cy);
        const int z0 = __reduce_min_sync(0xffffffffu, cz), z1 = __reduce_max_sync(0xffffffffu, cz);
        const int32_t sBase = B.cellStart[R.cellBase];
        const int32_t sEnd = B.cellStart[R.cellBase + R.gn[0] * R.gn[1] * R.gn[2]];
        const int az0 = max(z0 - 1, 0), az1 = min(z1 + 1, R.gn[2] - 1);
        int32_t cnt = 0, next = 0;  // first j-cluster not visited yet
        for (int ax = max(x0 - 1, 0); ax <= min(x1 + 1, R.gn[0] - 1); ++ax)
        {
            for (int ay = max(y0 - 1, 0); ay <= min(y1 + 1, R.gn[1] - 1); ++ay)
            {
                const int32_t c0 = R.cellBase + (ax * R.gn[1] + ay) * R.gn[2];
                const int32_t s0 = B.cellStart[c0 + az0], s1 = B.cellStart[c0 + az1 + 1];
                if (s1 <= s0) continue;
                const int32_t k1 = (s1 - 1 - sBase) / CLUSTER_J;
                for (int32_t k = max((s0 - sBase) / CLUSTER_J, next); k <= k1; ++k)
                {
                    const int32_t s = sBase + CLUSTER_J * k + sb;
                    bool keep = false, rev = false;
                    if (rowValid && s < sEnd)
                    {
                        const float4 q = B.spos[s];
                        const int32_t j = __float_as_int(q.w);
                        keep = j != i && !(rowCG && fabsf(q.x - cxRel) > deepCG);
                        if (keep)
                        {
                            const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
                            const float d2f = dx * dx + dy * dy + dz * dz;
                            keep = !(d2f > B.listRsqHi);
                            if (keep && !(d2f < B.listRsqLo))
                            {
                                const double4 pj = B.pos[j];
                                const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
                                const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)),
                                                            __dmul_rn(ddz, ddz));
                                keep = d2 <= B.listRsq;
                            }
                        }
                        if (keep && j >= B.N && !lex_above(pi, B.pos[j]))
                        {
                            const uint32_t code = B.gShift[j - B.N];
#pragma unroll
                            for (int d = 0; d < 3; ++d)
                            {
                                const uint32_t cd = (code >> (2 * d)) & 3u;
                                if (cd == 1) keep = keep && (myImg & (2u << (2 * d)));
                                if (cd == 2) keep = keep && (myImg & (1u << (2 * d)));
                            }
                            rev = true;
                        }
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, keep);
                    const uint32_t rm = __ballot_sync(0xffffffffu, keep && rev);
                    if (m)
                    {
                        if (lane == 0 && cnt < B.listCapC)
                            B.clist[(int64_t)c * B.listCapC + cnt] =
                                make_int4(sBase + CLUSTER_J * k, (int32_t)m, (int32_t)rm, 0);
                        ++cnt;
                    }
                }
                next = k1 + 1;
            }
        }
        if (lane == 0)
        {
            B.countsC[c] = cnt < B.listCapC ? cnt : B.listCapC;
            if (cnt > B.listCapC)
            {
                atomicMax(&B.sc->maxCountC, cnt);
                atomicOr(&B.sc->overflow, FLAG_CLUSTER_LIST_OVERFLOW);
            }
        }
    }
}

// ------------------------------------------------------------ pair force --
__device__ __forceinline__ df df_shfl_xor(df v, int o)
{
    return {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}

__device__ __forceinline__ double to_d(df v) { return (double)v.h + (double)v.l; }

// CheckRegion's hybrid test on a double-float weight in [0, 1]
__device__ __forceinline__ bool is_hy_df(float2 v)
{
    const bool at = v.x > 1.0f || (v.x == 1.0f && v.y >= 0.0f);
    return !at && !(v.x <= 0.0f);
}

// double-float pair energy: u3 (ef1 u3 - ef2) - shift with u3 = r^-6, or
// inside the cap E(r_cap) - (r - r_cap) capCoeff - shift
__device__ __forceinline__ df energy_df(const df& r2, const LJDev& p)
{
    if (r2.h >= p.capSqrf)
    {
        const df u = df_rcp(r2);
        const df u3 = df_mul(df_sqr(u), u);
        const df t = df_add(df_mul(df{p.ef1f, p.ef1l}, u3), df{-p.ef2f, -p.ef2l});
        return df_add(df_mul(u3, t), df{-p.shiftf, -p.shiftl});
    }
    const df t = df_add(df_sqrt(r2), df{-p.capDistf, -p.capDistl});
    const df lin = df_mul(t, df{p.capCoeff_f, p.capCoeff_l});
    return df_add(df{p.eCapShh, p.eCapShl}, df{-lin.h, -lin.l});
}

// x of i's image: side 1 = x - L, side 2 = x + L
__device__ __forceinline__ double image_x(double x, const RepDev& R, int side)
{
    return side == 1 ? __dsub_rn(x, R.L[0]) : __dadd_rn(x, R.L[0]);
}

// weights of i's image in x (side 1: -L, side 2: +L): those of i's ghost
// with that pure x shift (lambda depends on x only)
__device__ __forceinline__ void image_weights(const BDev& B, const RepDev& R, int32_t i, int side, double& l,
                                              double& m, double& g)
{
    const int2 xi = B.xImg[i];
    const int32_t slot = side == 1 ? xi.x : xi.y;
    if (slot >= 0)
    {
        const double4 w = B.lam[slot];
        l = w.x;
        m = w.y;
        g = w.z;
        return;
    }
    slab_eval(R.slab, image_x(B.pos[i].x, R, side), l, m, g);
}

struct RowOut
{
    double fx, fy, fz;  // pair force on the molecule
    double vsum;        // sum of V_ij of pairs with a hybrid member, own slot = the molecule itself
    double comp;        // the same, only pairs whose own slot is hybrid with a valid bin
    double imgFx;       // drift force from pairs whose own slot is an image of the molecule (FP64 form)
    double vImgM, vImgP;  // mixed form: V_ij sums of those pairs per image (-L, +L in x)
    double energy;      // sum of e w over the row (each pair is seen from both sides), FP64 form
    float fenergy;      // the same in the mixed form (FP32 pair energies)
};

// One row (local molecule i), lanes `sub` of TPR.  Returns this lane's
// partial sums.  CL: the row is row `lane >> 2` of i-cluster c (-1: none) and
// the lane takes slot `sub` of each j-cluster whose mask has bit `lane`.
template <bool MIXED, int TPR, bool CL = false>
__device__ __forceinline__ RowOut row_force(const BDev& B, int32_t i, int sub, bool sampling, int32_t c = -1,
                                            int lane = 0)
{
    const RepDev& R = B.reps[B.slotRep[i]];
    const double4 la = B.lam[i];  // lambda, modulated, grad x
    const double4 pi = B.pos[i];
    float4 hi_i, lo_i;
    if (MIXED)
    {
        hi_i = B.hi[i];
        lo_i = B.lo[i];
    }
    const float2 ltA = MIXED ? B.lamtf[i] : make_float2(0.f, 0.f);
    // weights of i's images in x (replicas whose slab reaches the ghost layer)
    int2 xImg = make_int2(-1, -1);
    float2 imgFM = ltA, imgFP = ltA;
    if (!R.consistent)
    {
        xImg = B.xImg[i];
        if (MIXED)
        {
            if (xImg.x >= 0) imgFM = B.lamtf[xImg.x];
            if (xImg.y >= 0) imgFP = B.lamtf[xImg.y];
        }
    }
    df fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, vs{0.f, 0.f}, cs{0.f, 0.f};
    df vImgM{0.f, 0.f}, vImgP{0.f, 0.f};  // mixed form: V_ij sums of pairs acting through i's -L / +L image
    double dfx = 0.0, dfy = 0.0, dfz = 0.0, dvs = 0.0, dcs = 0.0;
    double imgFx = 0.0, energy = 0.0;
    float fenergy = 0.0f;
    const int binAlpha = is_hy(la.y) ? comp_bin(la.x) : -1;
    float ffx = 0.0f, ffy = 0.0f, ffz = 0.0f, vsF = 0.0f, csF = 0.0f;  // FP32 sums of the far pairs
    auto pair_entry = [&](const int32_t entry) {
        const bool rev = entry < 0;
        const int32_t j = entry & 0x7fffffff;
        // own slot (the molecule or one of its images) and partner slot weights
        bool ownIsSelf = true;
        double ownLam = la.x, ownMod = la.y, ownGx = la.z;
        double partMod = 0.0;
        float2 partModF = make_float2(0.f, 0.f);
        if (MIXED)
            partModF = B.lamtf[j];
        else
            partMod = B.lamt[j];
        float2 ownImgF = ltA;
        int imgSide = 0;  // mixed form: 1 / 2 when the own slot is i's -L / +L image in x
        if (rev && !R.consistent)
        {
            // the pair acts with the weights of (source, image of i): the
            // image's weights are those of i's ghost with the opposite shift
            const int32_t g = j - B.N;
            const int32_t src = B.gSrc[g];
            if (MIXED)
                partModF = B.lamtf[src];
            else
                partMod = B.lamt[src];
            const uint32_t code = B.gShift[g];
            if (code & 3u)
            {
                // the own slot is i's image with the opposite x shift
                const int side = (code & 3u) == 1 ? 1 : 2;
                const int32_t slot = side == 1 ? xImg.x : xImg.y;
                if (MIXED)
                {
                    // double work stays out of the pair loop: the image's
                    // drift term is summed per image and applied per row
                    imgSide = side;
                    if (slot >= 0)
                    {
                        ownImgF = side == 1 ? imgFM : imgFP;
                    }
                    else
                    {
                        slab_eval(R.slab, image_x(pi.x, R, side), ownLam, ownMod, ownGx);
                        ownImgF = make_float2((float)ownMod, (float)(ownMod - (double)(float)ownMod));
                    }
                }
                else if (slot >= 0)
                {
                    const double4 li = B.lam[slot];
                    ownLam = li.x;
                    ownMod = li.y;
                    ownGx = li.z;
                }
                else
                {
                    slab_eval(R.slab, image_x(pi.x, R, side), ownLam, ownMod, ownGx);
                }
                ownIsSelf = false;
            }
        }
        if (MIXED)
        {
            const float2 ownF = ownImgF;
            if (ownF.x <= 0.0f && partModF.x <= 0.0f) return;  // both coarse grained: ideal gas
            const float4 hj = B.hi[j], lj = B.lo[j];
            if (B.farF32 && ownIsSelf)
            {
                // beyond r_split: plain FP32 (the LJ pair force is at most
                // |F(r_split)| there, 1.67 epsilon/sigma at 1.4 sigma); the
                // weights enter with their FP32 heads
                const float dx = (hi_i.x - hj.x) + (lo_i.x - lj.x);
                const float dy = (hi_i.y - hj.y) + (lo_i.y - lj.y);
                const float dz = (hi_i.z - hj.z) + (lo_i.z - lj.z);
                const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
                if (r2 > B.rc2.h * 1.0000005f) return;
                if (r2 >= B.rsplitSq && r2 < B.rc2.h * 0.9999995f)
                {
                    const float u = __fdividef(1.0f, r2);
                    const float u3 = u * u * u;
                    const float ff = u3 * u * __fmaf_rn(B.lj.ff1h, u3, -B.lj.ff2h);
                    const float e = __fmaf_rn(u3, __fmaf_rn(B.lj.ef1f, u3, -B.lj.ef2f), -B.lj.shiftf);
                    const bool bothAT =
                        ownF.x == 1.0f && ownF.y == 0.0f && partModF.x == 1.0f && partModF.y == 0.0f;
                    const float w = bothAT ? 1.0f : 0.5f * (ownF.x + partModF.x);
                    const float ffw = ff * w;
                    ffx = __fmaf_rn(dx, ffw, ffx);
                    ffy = __fmaf_rn(dy, ffw, ffy);
                    ffz = __fmaf_rn(dz, ffw, ffz);
                    if (is_hy_df(ownF) || is_hy_df(partModF))
                    {
                        const float V = 0.5f * e;  // V_ij = e/2 drives the drift force
                        vsF += V;
                        if (sampling && binAlpha != -1) csF += V;
                    }
                    fenergy = __fmaf_rn(e, w, fenergy);
                    return;
                }
            }
            PairMixed q;
            if (!pair_mixed(hi_i, lo_i, hj, lj, B.lj, B.rc2, q)) return;
            const bool hyPair = is_hy_df(ownF) || is_hy_df(partModF);
            // weighting = (lambda~_own + lambda~_partner) / 2 as a double-float
            const bool bothAT = ownF.x == 1.0f && ownF.y == 0.0f && partModF.x == 1.0f && partModF.y == 0.0f;
            df ffw = q.ff;
            if (!bothAT)
            {
                df w = df_add(df{ownF.x, ownF.y}, df{partModF.x, partModF.y});
                w.h *= 0.5f;
                w.l *= 0.5f;
                ffw = df_mul(q.ff, w);
            }
            df_acc_prod(fx, q.dh.x, q.dl.x, ffw);
            df_acc_prod(fy, q.dh.y, q.dl.y, ffw);
            df_acc_prod(fz, q.dh.z, q.dl.z, ffw);
            if (hyPair)
            {
                // V_ij = e/2 in double-float (it drives the drift force)
                const df ed = energy_df(df{q.r2h, q.r2l}, B.lj);
                const df V = {0.5f * ed.h, 0.5f * ed.l};
                if (ownIsSelf)
                {
                    vs = df_add(vs, V);
                    if (sampling && binAlpha != -1) cs = df_add(cs, V);
                }
                else if (imgSide == 1)
                {
                    vImgM = df_add(vImgM, V);  // drift and sampling of the image: per row, below
                }
                else
                {
                    vImgP = df_add(vImgP, V);
                }
            }
            fenergy = __fmaf_rn(q.e, bothAT ? 1.0f : 0.5f * (ownF.x + partModF.x), fenergy);
        }
        else
        {
            if (ownMod <= 0.0 && partMod <= 0.0) return;  // both coarse grained: ideal gas
            const double4 pj = B.pos[j];
            const double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            // explicit roundings: the same bits in every kernel that inlines
            // this body
            const double distSqr = __fma_rn(dx, dx, __fma_rn(dy, dy, __dmul_rn(dz, dz)));
            if (distSqr > B.rcSqr) return;
            const bool hyPair = is_hy(ownMod) || is_hy(partMod);
            double ff, e;
            lj_eval_fp64(B.lj, distSqr, ff, e);
            const double weighting = 0.5 * (ownMod + partMod);
            const double ffactor = ff * weighting;
            dfx = fma(dx, ffactor, dfx);
            dfy = fma(dy, ffactor, dfy);
            dfz = fma(dz, ffactor, dfz);
            energy = fma(e, weighting, energy);
            if (hyPair)
            {
                const double Vij = 0.5 * e;
                if (ownIsSelf)
                {
                    dvs += Vij;
                    if (sampling && binAlpha != -1) dcs += Vij;
                }
                else
                {
                    imgFx = fma(-Vij, ownGx, imgFx);
                    if (sampling && is_hy(ownMod))
                    {
                        const int b = comp_bin(ownLam);
                        if (b != -1)
                            atomicAdd(reinterpret_cast<unsigned long long*>(B.compEnergy + B.slotRep[i] * COMP_BINS + b),
                                      (unsigned long long)llrint(Vij * COMP_SCALE));
                    }
                }
            }
        }
        };
    if (CL)
    {
        // every lane walks the cluster's row (uniform loop, broadcast loads)
        const int cntC = c >= 0 ? B.countsC[c] : 0;
        const int4* row = B.clist + (int64_t)(c >= 0 ? c : 0) * B.listCapC;
        for (int k = 0; k < cntC; ++k)
        {
            const int4 e = row[k];
            if (((uint32_t)e.y >> lane) & 1u)
            {
                const int32_t j = B.sorted[e.x + sub];
                pair_entry((((uint32_t)e.z >> lane) & 1u) ? (j | REVERSED) : j);
            }
        }
    }
    else
    {
        const int cnt = B.counts[i];
        const int64_t rowBase = mrmd_dev::nbr_row(i, B.listCap);
        for (int k = sub; k < cnt; k += TPR) pair_entry(B.nbrs[rowBase + 32 * (int64_t)k]);
    }
    if (MIXED && B.split)
    {
        const int cntF = B.countsF[i];
        const int64_t rowBaseF = mrmd_dev::nbr_row(i, B.listCapF);
        for (int k = sub; k < cntF; k += TPR) pair_entry(B.nbrsF[rowBaseF + 32 * (int64_t)k]);
    }
    if (MIXED)
    {
        df_acc(fx, ffx);
        df_acc(fy, ffy);
        df_acc(fz, ffz);
        df_acc(vs, vsF);
        df_acc(cs, csF);
    }
    // reduce the TPR lanes of the row (fixed butterfly: identical sums on every lane)
    RowOut o;
    if (MIXED)
    {
#pragma unroll
        for (int off = 1; off < TPR; off <<= 1)
        {
            fx = df_add(fx, df_shfl_xor(fx, off));
            fy = df_add(fy, df_shfl_xor(fy, off));
            fz = df_add(fz, df_shfl_xor(fz, off));
            vs = df_add(vs, df_shfl_xor(vs, off));
            cs = df_add(cs, df_shfl_xor(cs, off));
            vImgM = df_add(vImgM, df_shfl_xor(vImgM, off));
            vImgP = df_add(vImgP, df_shfl_xor(vImgP, off));
        }
        o.vImgM = to_d(vImgM);
        o.vImgP = to_d(vImgP);
        o.fx = to_d(fx);
        o.fy = to_d(fy);
        o.fz = to_d(fz);
        o.vsum = to_d(vs);
        o.comp = sampling ? to_d(cs) : 0.0;
    }
    else
    {
#pragma unroll
        for (int off = 1; off < TPR; off <<= 1)
        {
            dfx += __shfl_xor_sync(0xffffffffu, dfx, off);
            dfy += __shfl_xor_sync(0xffffffffu, dfy, off);
            dfz += __shfl_xor_sync(0xffffffffu, dfz, off);
            dvs += __shfl_xor_sync(0xffffffffu, dvs, off);
            dcs += __shfl_xor_sync(0xffffffffu, dcs, off);
        }
        o.fx = dfx;
        o.fy = dfy;
        o.fz = dfz;
        o.vsum = dvs;
        o.comp = dcs;
        o.vImgM = 0.0;
        o.vImgP = 0.0;
    }
#pragma unroll
    for (int off = 1; off < TPR; off <<= 1)
    {
        imgFx += __shfl_xor_sync(0xffffffffu, imgFx, off);
        if (MIXED)
            fenergy += __shfl_xor_sync(0xffffffffu, fenergy, off);
        else
            energy += __shfl_xor_sync(0xffffffffu, energy, off);
    }
    o.imgFx = imgFx;
    o.energy = energy;
    o.fenergy = fenergy;
    return o;
}

// Pair force of every local molecule (LJ_IdealGas.cpp:52-225 on a full
// list), then per molecule: drift-compensation force and sampling, TF apply
// (ThermodynamicForce.hpp:98-122), density sample (AxialDensityProfile.cpp:
// 36-47) and the velocity-Verlet post kick (VelocityVerlet.cpp:69-90).
// CL: one warp per i-cluster, 4 lanes per row (TPR = 4).
// One thread's share of the force for global thread index gtid (a warp's
// 32 lanes take 32 consecutive indices, aligned to 32).
template <bool MIXED, int TPR, bool CL>
__device__ __forceinline__ void force_body(const BDev& B, int64_t gtid)
{
    static_assert(!CL || TPR == CLUSTER_J, "the cluster layout has CLUSTER_J lanes per row");
    const bool sampling = B.sc->sampleComp != 0;
    const bool tfSample = B.sc->sampleTf != 0;
    int32_t i = (int32_t)(gtid / TPR);
    const int sub = (int)(gtid % TPR);
    bool valid = i < B.N;
    int32_t c = -1;
    if (CL)
    {
        const int32_t w = (int32_t)(gtid >> 5);
        const int a = (threadIdx.x & 31) / CLUSTER_J;
        c = w < B.numClusters ? w : -1;
        const int2 cl = c >= 0 ? B.clusters[c] : make_int2(0, 0);
        valid = c >= 0 && a < cl.y;
        i = valid ? cl.x + a : cl.x;
    }
    RowOut o = row_force<MIXED, TPR, CL>(B, valid ? i : 0, sub, sampling && valid, c, threadIdx.x & 31);
    int32_t r = valid ? B.slotRep[i] : -1;
    if (valid && sub == 0)
    {
        const RepDev& R = B.reps[r];
        const double4 la = B.lam[i];
        // molecule force: drift (-V_ij grad lambda) and compensation
        double fmx = fma(-o.vsum, la.z, o.imgFx);
        if (MIXED && (o.vImgM != 0.0 || o.vImgP != 0.0))
        {
            // pairs acting through i's images: drift force -V grad lambda of the
            // image and, on sampling runs, V into the image's compensation bin
#pragma unroll
            for (int side = 1; side <= 2; ++side)
            {
                const double v = side == 1 ? o.vImgM : o.vImgP;
                if (v == 0.0) continue;
                double l, m, g;
                image_weights(B, R, i, side, l, m, g);
                fmx = fma(-v, g, fmx);
                if (sampling && is_hy(m))
                {
                    const int b = comp_bin(l);
                    if (b != -1)
                        atomicAdd(reinterpret_cast<unsigned long long*>(B.compEnergy + r * COMP_BINS + b),
                                  (unsigned long long)llrint(v * COMP_SCALE));
                }
            }
        }
        if (is_hy(la.y))
        {
            const int b = comp_bin(la.x);
            if (b != -1)
            {
                fmx = fma(B.compMean[r * COMP_BINS + b], la.z, fmx);
                if (sampling)
                {
                    atomicAdd(B.compCounter + r * COMP_BINS + b, 1ull);
                    atomicAdd(reinterpret_cast<unsigned long long*>(B.compEnergy + r * COMP_BINS + b),
                              (unsigned long long)llrint(o.comp * COMP_SCALE));
                }
            }
        }
        double4 f = make_double4(o.fx, o.fy, o.fz, 0.0);
        f.x = __dadd_rn(f.x, fmx);
        const double4 x = B.pos[i];
        if (B.tfEnabled)
        {
            const int64_t b = (int64_t)floor((x.x - R.tfMin) * R.tfInvBin);
            if (b >= 0 && b < R.tfBins)
            {
                f.x = __dadd_rn(f.x, B.tfForce[R.tfBase + b]);
                if (tfSample) atomicAdd(B.tfDensity + R.tfBase + b, 1ull);
            }
        }
        double4 v = B.vel[i];
        kick_fma(v, f, B.dtHalfOverMass);
        B.vel[i] = v;
        B.force[i] = f;
    }
    // energy per replica: one atomic per warp when the warp's rows share a replica
    const int lane = threadIdx.x & 31;
    const int32_t r0 = __shfl_sync(0xffffffffu, r, 0);
    double* ring = B.energyRing + (int64_t)B.sc->ringSlot * B.R;
    const bool oneReplica = __all_sync(0xffffffffu, r == r0 || r == -1);
    if (MIXED)
    {
        float e = (sub == 0 && valid) ? 0.5f * o.fenergy : 0.0f;
        if (oneReplica)
        {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) e += __shfl_down_sync(0xffffffffu, e, off);
            if (lane == 0 && r0 >= 0) atomicAdd(ring + r0, (double)e);
        }
        else if (r >= 0 && e != 0.0f)
        {
            atomicAdd(ring + r, (double)e);
        }
    }
    else
    {
        double e = (sub == 0 && valid) ? 0.5 * o.energy : 0.0;
        if (oneReplica)
        {
            e = mrmd_dev::warp_sum(e);
            if (lane == 0 && r0 >= 0) atomicAdd(ring + r0, e);
        }
        else if (r >= 0 && e != 0.0)
        {
            atomicAdd(ring + r, e);
        }
    }
}

// 80 registers: six blocks of 128 threads per SM (86 registers gave five
// and an 8% slower step)
template <bool MIXED, int TPR, bool CL>
__global__ void __maxnreg__(80) k_b_force(BDev B)
{
    force_body<MIXED, TPR, CL>(B, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// pairs (mask bits) and cluster pairs of the cluster layout's rows
__global__ void k_b_cluster_stats(BDev B, unsigned long long* out)
{
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < B.numClusters; c += gridDim.x * blockDim.x)
    {
        const int n = B.countsC[c];
        unsigned long long bits = 0;
        for (int k = 0; k < n; ++k) bits += (unsigned long long)__popc((uint32_t)B.clist[(int64_t)c * B.listCapC + k].y);
        atomicAdd(out, bits);
        atomicAdd(out + 1, (unsigned long long)n);
    }
}

// ------------------------------------------------------------------ tail --
// The step decisions the tail reads (thread 0, before the counters advance).
struct TailShared
{
    unsigned long long step, run, samples;
    int compUpdate, tfUpdate;
};

__device__ __forceinline__ void tail_read(const BDev& B, TailShared& t)
{
    t.step = B.sc->step;
    t.run = B.sc->run;
    t.samples = B.sc->tfSamples + (unsigned long long)(B.sc->sampleTf != 0);  // including this step's sample
    t.compUpdate = B.compUpdate > 0 && (t.run % (unsigned long long)B.compUpdate) == 0;
    t.tfUpdate = B.tfEnabled && ((t.step + 1) % (unsigned long long)B.tfUpdateInterval) == 0 && t.samples > 0;
}

// Replica r's drift-compensation mean update (LJ_IdealGas.cpp:21-50, 253-255)
// and ThermodynamicForce update, by one block.
__device__ __forceinline__ void tail_replica(const BDev& B, int r, const TailShared& t)
{
    const RepDev& R = B.reps[r];
    if (t.compUpdate)
    {
        for (int k = threadIdx.x; k < COMP_BINS; k += blockDim.x)
        {
            const int64_t q = (int64_t)r * COMP_BINS + k;
            const double cnt = (double)B.compCounter[q];
            if (cnt < 0.5) continue;
            const double e = ((double)B.compEnergy[q] / COMP_SCALE) / cnt;
            B.compMean[q] = (10.0 * B.compMean[q] + e) / (10.0 + 1.0);
            B.compEnergy[q] = 0;
            B.compCounter[q] = 0;
        }
    }
    if (t.tfUpdate)
    {
        double* d = B.tfWork + R.tfBase;
        for (int k = threadIdx.x; k < R.tfBins; k += blockDim.x)
        {
            d[k] = (double)B.tfDensity[R.tfBase + k];
            B.tfDensity[R.tfBase + k] = 0ull;
        }
        __syncthreads();
        UpdateArgs A{};
        A.density = d;
        A.force = B.tfForce + R.tfBase;
        A.smooth = B.tfWork + B.totalBins + R.tfBase;
        A.grad = B.tfWork + 2 * (int64_t)B.totalBins + R.tfBase;
        A.forceFactor = B.tfFF;
        A.numBins = R.tfBins;
        A.numTypes = 1;
        A.binSize = R.tfBinSize;
        A.inverseBinSize = R.tfInvBin;
        A.min = R.tfMin;
        A.normalization = 1.0 / (R.tfBinVolume * (double)t.samples);
        A.sigma = B.tfSigma;
        A.range = B.tfRange;
        A.enforceSymmetry = 0;
        A.periodic = 1;
        A.usePred = 0;
        tf_update_block(A);
    }
}

// The step counters and the displacement bookkeeping (one thread, after
// every replica's tail).
__device__ __forceinline__ void tail_counters(const BDev& B, int rebuild, const TailShared& t)
{
    Scalars* s = B.sc;
    s->tfSamples = t.tfUpdate ? 0ull : t.samples;
    // on a rebuild step the pre-force displacement is measured against
    // the previous list, which this step no longer uses
    if (rebuild)
    {
        s->maxDisp = 0.0;
    }
    else
    {
        const double d = sqrt(s->dispStep);
        s->maxDisp = fmax(s->maxDisp, d);
        if (d >= B.halfSkin) s->flags |= FLAG_UNSAFE_INTERVAL;
    }
    s->dispStep = 0.0;
    s->run = t.run + 1;
    s->step = t.step + 1;
    set_step_flags(*s, t.step + 1, t.run + 1, B.ring, B.compSampling, B.tfEnabled, B.tfSampleInterval);
}

// One block per replica; the last block to finish advances the counters.
__global__ void k_b_tail(BDev B, int rebuild)
{
    __shared__ TailShared t;
    if (threadIdx.x == 0) tail_read(B, t);
    __syncthreads();
    tail_replica(B, blockIdx.x, t);
    __syncthreads();
    __threadfence();
    if (threadIdx.x == 0)
    {
        const unsigned int ticket = atomicAdd(&B.sc->done, 1u);
        if (ticket == gridDim.x - 1)
        {
            __threadfence();
            tail_counters(B, rebuild, t);
            B.sc->done = 0u;
        }
    }
}

// ------------------------------------------------------ persistent steps --
// A grid-wide barrier with a wall-clock limit: the blocks of a cooperative
// launch (all resident) arrive on a counter; the last one resets it and
// advances the generation the others wait on.  A wait longer than limitNs,
// or an error raised by another block, ends with `error` set and false
// returned: the caller returns, and the host reads the error.
struct GridBar
{
    unsigned* count;
    unsigned* gen;
    int32_t* error;
    unsigned long long limitNs;
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// every thread of every block; skip (tests only): this block never arrives
__device__ bool grid_sync(const GridBar& gb, bool skip = false)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        volatile unsigned* gen = gb.gen;
        volatile int32_t* err = gb.error;
        const unsigned g = *gen;
        __threadfence();
        bool released = false;
        if (!skip && atomicAdd(gb.count, 1u) == gridDim.x - 1)
        {
            *gb.count = 0u;
            __threadfence();
            atomicAdd(gb.gen, 1u);
            released = true;
        }
        bool good = *err == 0;
        if (!released && good)
        {
            const unsigned long long t0 = global_ns();
            while (*gen == g)
            {
                if (*err != 0)
                {
                    good = false;
                    break;
                }
                if (global_ns() - t0 > gb.limitNs)
                {
                    atomicExch(gb.error, 1);
                    good = false;
                    break;
                }
                __nanosleep(200);
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// `count` steps without rebuild in one cooperative launch: the four phases
// of step() (pre, ghost update, force, tail) separated by grid barriers,
// the same arithmetic per molecule, ghost, row and replica.
template <bool MIXED, int TPR, bool CL>
__global__ void __maxnreg__(80) k_b_steps(BDev B, int count, GridBar gb)
{
    __shared__ TailShared t;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t threads = CL ? (int64_t)B.numClusters * 32 : (int64_t)B.N * TPR;
    for (int k = 0; k < count; ++k)
    {
        pre_body<MIXED>(B, 0, tid, stride);
        if (!grid_sync(gb)) return;
        ghost_update_body<MIXED>(B, tid, stride);
        if (!grid_sync(gb)) return;
        for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < threads; base += stride)
            force_body<MIXED, TPR, CL>(B, base + threadIdx.x);
        if (!grid_sync(gb)) return;
        if (threadIdx.x == 0) tail_read(B, t);
        __syncthreads();
        for (int r = blockIdx.x; r < B.R; r += gridDim.x)
        {
            tail_replica(B, r, t);
            __syncthreads();
        }
        if (!grid_sync(gb)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) tail_counters(B, 0, t);
        if (!grid_sync(gb)) return;
    }
}

// `rounds` barriers; block `skipBlock` (>= 0, tests only) never arrives.
__global__ void k_grid_sync_test(GridBar gb, int rounds, int skipBlock)
{
    for (int k = 0; k < rounds; ++k)
        if (!grid_sync(gb, (int)blockIdx.x == skipBlock)) return;
}
}  // namespace

// ================================================================== host ==

namespace mrmd_batch_impl
{
void drop_graph(mrmd_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// (Re)size the ghost-dependent and list buffers.
int set_capacity(mrmd_ctx* ctx, mrmd_batch* b, int32_t gCap, int32_t listCap, int32_t listCapF, int32_t listCapC)
{
    BDev& B = b->B;
    const int64_t N = b->N;
    if (gCap != B.gCap)
    {
        const int64_t o = N + B.gCap, n = N + gCap;
        MRMD_TRY(grow(ctx, B.pos, o, n));
        MRMD_TRY(grow(ctx, B.slotRep, o, n));
        MRMD_TRY(grow(ctx, B.lam, o, n));
        MRMD_TRY(grow(ctx, B.lamt, o, n));
        MRMD_TRY(grow(ctx, B.lamtf, o, n));
        MRMD_TRY(grow(ctx, B.hi, o, n));
        MRMD_TRY(grow(ctx, B.lo, o, n));
        MRMD_TRY(grow(ctx, B.cellOf, 0, n));
        MRMD_TRY(grow(ctx, B.unordered, 0, n));
        MRMD_TRY(grow(ctx, B.sorted, 0, n));
        MRMD_TRY(grow(ctx, B.spos, 0, n));
        MRMD_TRY(grow(ctx, B.gSrc, 0, (int64_t)gCap));
        MRMD_TRY(grow(ctx, B.gShift, 0, (int64_t)gCap));
        B.gCap = gCap;
        drop_graph(b);
    }
    if (listCap != B.listCap)
    {
        const int64_t tiles = div_up(N, 32);
        MRMD_TRY(grow(ctx, B.nbrs, 0, tiles * 32 * (int64_t)listCap));
        B.listCap = listCap;
        drop_graph(b);
    }
    if (listCapF >= 0 && listCapF != B.listCapF)
    {
        const int64_t tiles = div_up(N, 32);
        MRMD_TRY(grow(ctx, B.nbrsF, 0, tiles * 32 * (int64_t)std::max(listCapF, 1)));
        B.listCapF = listCapF;
        drop_graph(b);
    }
    if (listCapC >= 0 && listCapC != B.listCapC)
    {
        MRMD_TRY(grow(ctx, B.clist, 0, (int64_t)B.numClusters * std::max(listCapC, 1)));
        B.listCapC = listCapC;
        drop_graph(b);
    }
    return MRMD_OK;
}

// the list layout of the tuning: near/far rows for the mixed form only, FP32
// far pairs in the mixed form's near/far and cluster layouts; the cluster
// rows are allocated when the layout is first used (a guess that the
// overflow recovery grows)
int apply_layout(mrmd_ctx* ctx, mrmd_batch* b)
{
    const int32_t layout = b->cfg.tuning.listLayout;
    const bool mixed = b->cfg.precision == MRMD_PREC_MIXED;
    b->B.split = (mixed && layout == LAYOUT_NEAR_FAR) ? 1 : 0;
    b->B.farF32 = (mixed && (layout == LAYOUT_NEAR_FAR || layout == LAYOUT_CLUSTER)) ? 1 : 0;
    if (layout == LAYOUT_CLUSTER && b->B.listCapC == 0)
    {
        const int32_t c0 = b->cfg.initialMaxNeighbors > 0 ? (int32_t)b->cfg.initialMaxNeighbors : 96;
        return set_capacity(ctx, b, b->B.gCap, b->B.listCap, -1, c0);
    }
    return MRMD_OK;
}

// Cell binning of the locals (withGhosts = 0) or of every slot.
int cell_pass(mrmd_ctx* ctx, mrmd_batch* b, int withGhosts)
{
    BDev& B = b->B;
    const int64_t n = withGhosts ? (int64_t)b->N + B.gCap : b->N;
    MRMD_CUDA(ctx, cudaMemsetAsync(B.cellStart, 0, sizeof(int32_t) * (size_t)(b->totalCells + 1), ctx->stream));
    MRMD_CUDA(ctx, cudaMemsetAsync(B.cursor, 0, sizeof(int32_t) * (size_t)(b->totalCells + 1), ctx->stream));
    const unsigned g = grid_for(ctx, n, TB);
    k_b_cell_count<<<g, TB, 0, ctx->stream>>>(B, withGhosts);
    MRMD_TRY(after_launch(ctx, "batch cell_count"));
    MRMD_TRY(scan_exclusive_i32(ctx, B.cellStart, B.cellStart, b->totalCells + 1, nullptr));
    k_b_cell_scatter<<<g, TB, 0, ctx->stream>>>(B, withGhosts);
    MRMD_TRY(after_launch(ctx, "batch cell_scatter"));
    k_b_cell_rank<<<g, TB, 0, ctx->stream>>>(B, withGhosts);
    return after_launch(ctx, "batch cell_rank");
}

template <bool M>
int rebuild_t(mrmd_ctx* ctx, mrmd_batch* b, bool sort)
{
    BDev& B = b->B;
    const unsigned gN = grid_for(ctx, b->N, TB);
    if (sort)
    {
        MRMD_TRY(cell_pass(ctx, b, 0));
        k_b_sort_gather<<<gN, TB, 0, ctx->stream>>>(B);
        MRMD_TRY(after_launch(ctx, "batch sort_gather"));
        k_b_sort_store<M><<<gN, TB, 0, ctx->stream>>>(B);
        MRMD_TRY(after_launch(ctx, "batch sort_store"));
    }
    k_b_ghost_count<<<gN, TB, 0, ctx->stream>>>(B);
    MRMD_TRY(after_launch(ctx, "batch ghost_count"));
    MRMD_TRY(scan_exclusive_i32(ctx, B.gCount, B.gCount, b->N, &B.sc->numGhost));
    k_b_ghost_write<M><<<gN, TB, 0, ctx->stream>>>(B);
    MRMD_TRY(after_launch(ctx, "batch ghost_write"));
    MRMD_TRY(cell_pass(ctx, b, 1));
    if (b->cfg.tuning.listLayout == LAYOUT_CLUSTER)
    {
        k_b_build_clusters<<<grid_for(ctx, (int64_t)B.numClusters * 32, 128, 16), 128, 0, ctx->stream>>>(B);
        return after_launch(ctx, "batch build_clusters");
    }
    k_b_build_list<<<grid_for(ctx, b->N, 128, 16), 128, 0, ctx->stream>>>(B);
    return after_launch(ctx, "batch build_list");
}

int rebuild(mrmd_ctx* ctx, mrmd_batch* b, bool sort)
{
    return b->cfg.precision == MRMD_PREC_MIXED ? rebuild_t<true>(ctx, b, sort) : rebuild_t<false>(ctx, b, sort);
}

template <bool M, int TPR, bool CL = false>
int force_t(mrmd_ctx* ctx, mrmd_batch* b)
{
    const int bs = b->cfg.tuning.blockSize;
    const int64_t threads = CL ? (int64_t)b->B.numClusters * 32 : (int64_t)b->N * TPR;
    k_b_force<M, TPR, CL><<<(unsigned)div_up(threads, bs), bs, 0, ctx->stream>>>(b->B);
    return after_launch(ctx, "batch force");
}

template <bool M>
int force_m(mrmd_ctx* ctx, mrmd_batch* b)
{
    if (b->cfg.tuning.listLayout == LAYOUT_CLUSTER) return force_t<M, CLUSTER_J, true>(ctx, b);
    switch (b->cfg.tuning.threadsPerRow)
    {
        case 1: return force_t<M, 1>(ctx, b);
        case 2: return force_t<M, 2>(ctx, b);
        case 4: return force_t<M, 4>(ctx, b);
        case 8: return force_t<M, 8>(ctx, b);
        default: return set_error(ctx, MRMD_ERR_ARG, "threadsPerRow must be 1, 2, 4 or 8");
    }
}

bool is_rebuild(const mrmd_batch* b, int64_t st) { return st % b->cfg.tuning.rebuildInterval == 0; }

bool is_sort(const mrmd_batch* b, int64_t st)
{
    const int64_t se = b->cfg.tuning.sortEvery;
    return se > 0 && is_rebuild(b, st) && (st / b->cfg.tuning.rebuildInterval) % se == 0;
}

int derive_locals(mrmd_ctx* ctx, mrmd_batch* b)
{
    const unsigned g = grid_for(ctx, b->N, TB);
    if (b->cfg.precision == MRMD_PREC_MIXED)
        k_b_derive<true><<<g, TB, 0, ctx->stream>>>(b->B);
    else
        k_b_derive<false><<<g, TB, 0, ctx->stream>>>(b->B);
    return after_launch(ctx, "batch derive");
}

int update_ghosts(mrmd_ctx* ctx, mrmd_batch* b)
{
    const unsigned g = grid_for(ctx, b->B.gCap, TB);
    if (b->cfg.precision == MRMD_PREC_MIXED)
        k_b_ghost_update<true><<<g, TB, 0, ctx->stream>>>(b->B);
    else
        k_b_ghost_update<false><<<g, TB, 0, ctx->stream>>>(b->B);
    return after_launch(ctx, "batch ghost_update");
}

int eval_forces(mrmd_ctx* ctx, mrmd_batch* b)
{
    MRMD_TRY(derive_locals(ctx, b));
    MRMD_TRY(rebuild_checked(ctx, b, false));
    return b->cfg.precision == MRMD_PREC_MIXED ? force_m<true>(ctx, b) : force_m<false>(ctx, b);
}

int rebuild_checked(mrmd_ctx* ctx, mrmd_batch* b, bool sort)
{
    BDev& B = b->B;
    for (int attempt = 0;; ++attempt)
    {
        MRMD_CUDA(ctx, cudaMemsetAsync(&B.sc->overflow, 0, sizeof(uint32_t), ctx->stream));
        MRMD_TRY(rebuild(ctx, b, sort));
        MRMD_CUDA(ctx, cudaMemcpyAsync(b->hSc, B.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const uint32_t f = b->hSc->overflow;
        if (!f) return MRMD_OK;
        if (attempt >= 4) return set_error(ctx, MRMD_ERR_NLIST_OVERFLOW, "batch buffers kept overflowing");
        int32_t gCap = B.gCap, lCap = B.listCap, fCap = B.listCapF, cCap = B.listCapC;
        if (f & FLAG_GHOST_OVERFLOW) gCap = b->hSc->numGhost + b->hSc->numGhost / 4 + 1024;
        if (f & FLAG_LIST_OVERFLOW) lCap = b->hSc->maxCount + b->hSc->maxCount / 5 + 8;
        if (f & FLAG_FAR_LIST_OVERFLOW) fCap = b->hSc->maxCountF + b->hSc->maxCountF / 5 + 8;
        if (f & FLAG_CLUSTER_LIST_OVERFLOW) cCap = b->hSc->maxCountC + b->hSc->maxCountC / 5 + 8;
        MRMD_TRY(set_capacity(ctx, b, gCap, lCap, fCap, cCap));
        b->recoveries++;
        sort = false;  // the locals are already in cell order
    }
}

// One step, asynchronously.  With checkRebuild the rebuild is verified on the
// host (one synchronisation) and repeated with larger buffers on overflow.
int step(mrmd_ctx* ctx, mrmd_batch* b, int64_t st, bool checkRebuild)
{
    BDev& B = b->B;
    const bool M = b->cfg.precision == MRMD_PREC_MIXED;
    const bool reb = is_rebuild(b, st) || b->needRebuild;
    b->needRebuild = false;
    const unsigned gN = grid_for(ctx, b->N, TB);
    if (M)
        k_b_pre<true><<<gN, TB, 0, ctx->stream>>>(B, reb ? 1 : 0);
    else
        k_b_pre<false><<<gN, TB, 0, ctx->stream>>>(B, reb ? 1 : 0);
    MRMD_TRY(after_launch(ctx, "batch pre"));
    if (reb)
    {
        if (checkRebuild)
            MRMD_TRY(rebuild_checked(ctx, b, is_sort(b, st)));
        else
            MRMD_TRY(rebuild(ctx, b, is_sort(b, st)));
        b->rebuilds++;
    }
    else
    {
        if (M)
            k_b_ghost_update<true><<<grid_for(ctx, B.gCap, TB), TB, 0, ctx->stream>>>(B);
        else
            k_b_ghost_update<false><<<grid_for(ctx, B.gCap, TB), TB, 0, ctx->stream>>>(B);
        MRMD_TRY(after_launch(ctx, "batch ghost_update"));
    }
    MRMD_TRY(M ? force_m<true>(ctx, b) : force_m<false>(ctx, b));
    k_b_tail<<<(unsigned)b->R, TB, 0, ctx->stream>>>(B, reb ? 1 : 0);
    return after_launch(ctx, "batch tail");
}

int snap_alloc(mrmd_ctx* ctx, const mrmd_batch* b, Snap& s)
{
    const int64_t N = b->N, nb = std::max<int64_t>(b->totalBins, 1), nc = (int64_t)b->R * COMP_BINS;
    MRMD_TRY(grow(ctx, s.pos, 0, N));
    MRMD_TRY(grow(ctx, s.vel, 0, N));
    MRMD_TRY(grow(ctx, s.force, 0, N));
    MRMD_TRY(grow(ctx, s.mass, 0, N));
    MRMD_TRY(grow(ctx, s.orig, 0, N));
    MRMD_TRY(grow(ctx, s.tfForce, 0, nb));
    MRMD_TRY(grow(ctx, s.tfDensity, 0, nb));
    MRMD_TRY(grow(ctx, s.compE, 0, nc));
    MRMD_TRY(grow(ctx, s.compC, 0, nc));
    MRMD_TRY(grow(ctx, s.compM, 0, nc));
    return grow(ctx, s.sc, 0, (int64_t)1);
}

void snap_free(Snap& s)
{
    void* ptrs[] = {s.pos, s.vel, s.force, s.mass, s.orig, s.tfForce, s.tfDensity, s.compE, s.compC, s.compM, s.sc};
    for (void* p : ptrs) dfree(p);
    s = Snap{};
}

// save (live -> s) or restore (s -> live)
int snapshot(mrmd_ctx* ctx, mrmd_batch* b, Snap& sn, bool save)
{
    BDev& B = b->B;
    const size_t N = (size_t)b->N, nb = (size_t)b->totalBins, nc = (size_t)b->R * COMP_BINS;
    auto cp = [&](void* snap, void* live, size_t bytes) {
        if (bytes == 0) return (int)MRMD_OK;
        return check_cuda(ctx,
                          cudaMemcpyAsync(save ? snap : live, save ? live : snap, bytes, cudaMemcpyDeviceToDevice,
                                          ctx->stream),
                          "batch snapshot");
    };
    MRMD_TRY(cp(sn.pos, B.pos, sizeof(double4) * N));
    MRMD_TRY(cp(sn.vel, B.vel, sizeof(double4) * N));
    MRMD_TRY(cp(sn.force, B.force, sizeof(double4) * N));
    MRMD_TRY(cp(sn.mass, B.mass, sizeof(double) * N));
    MRMD_TRY(cp(sn.orig, B.orig, sizeof(int32_t) * N));
    MRMD_TRY(cp(sn.tfForce, B.tfForce, sizeof(double) * nb));
    MRMD_TRY(cp(sn.tfDensity, B.tfDensity, sizeof(unsigned long long) * nb));
    MRMD_TRY(cp(sn.compE, B.compEnergy, sizeof(long long) * nc));
    MRMD_TRY(cp(sn.compC, B.compCounter, sizeof(unsigned long long) * nc));
    MRMD_TRY(cp(sn.compM, B.compMean, sizeof(double) * nc));
    MRMD_TRY(cp(sn.sc, B.sc, sizeof(Scalars)));
    return MRMD_OK;
}

// Wall-clock limit of one grid-barrier wait of the persistent step kernel:
// far above any phase of a step (milliseconds), short enough to give the
// GPU back quickly when a block never arrives.
constexpr unsigned long long SYNC_LIMIT_NS = 2000000000ull;

// A cooperative launch of the kernel with every block resident (blocks per
// SM from the occupancy calculator), captured like any launch.
template <typename... A>
int cooperative_launch(mrmd_ctx* ctx, void (*kernel)(A...), int blockSize, const char* what, A... args)
{
    int perSM = 0;
    MRMD_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, blockSize, 0));
    if (perSM < 1) return set_error(ctx, MRMD_ERR_CAPACITY, "%s: no block of %d threads fits an SM", what, blockSize);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(perSM * ctx->numSMs));
    cfg.blockDim = dim3((unsigned)blockSize);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    MRMD_CUDA(ctx, cudaLaunchKernelEx(&cfg, kernel, args...));
    return after_launch(ctx, what);
}

template <bool M, int TPR, bool CL = false>
int persistent_t(mrmd_ctx* ctx, mrmd_batch* b, int count)
{
    // a fresh barrier (count, generation); the error word is cleared by the
    // host before each graph launch and read after it
    MRMD_CUDA(ctx, cudaMemsetAsync(b->dSync, 0, 2 * sizeof(unsigned), ctx->stream));
    const GridBar gb{b->dSync, b->dSync + 1, reinterpret_cast<int32_t*>(b->dSync + 2), SYNC_LIMIT_NS};
    return cooperative_launch(ctx, k_b_steps<M, TPR, CL>, b->cfg.tuning.blockSize, "batch persistent steps", b->B,
                              count, gb);
}

template <bool M>
int persistent_m(mrmd_ctx* ctx, mrmd_batch* b, int count)
{
    if (b->cfg.tuning.listLayout == LAYOUT_CLUSTER) return persistent_t<M, CLUSTER_J, true>(ctx, b, count);
    switch (b->cfg.tuning.threadsPerRow)
    {
        case 1: return persistent_t<M, 1>(ctx, b, count);
        case 2: return persistent_t<M, 2>(ctx, b, count);
        case 4: return persistent_t<M, 4>(ctx, b, count);
        case 8: return persistent_t<M, 8>(ctx, b, count);
        default: return set_error(ctx, MRMD_ERR_ARG, "threadsPerRow must be 1, 2, 4 or 8");
    }
}

// `count` steps without rebuild in one persistent launch
int persistent_steps(mrmd_ctx* ctx, mrmd_batch* b, int count)
{
    return b->cfg.precision == MRMD_PREC_MIXED ? persistent_m<true>(ctx, b, count)
                                               : persistent_m<false>(ctx, b, count);
}

int capture(mrmd_ctx* ctx, mrmd_batch* b, int64_t st0)
{
    drop_graph(b);
    const int64_t P = b->cfg.tuning.graphSteps;
    MRMD_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = ctx->launches, r0 = b->rebuilds;
    int rc = MRMD_OK;
    if (b->cfg.tuning.persistent)
    {
        // each rebuild step on its own, then the steps up to the next rebuild
        // in one cooperative launch (P is a multiple of the rebuild interval)
        const int64_t K = b->cfg.tuning.rebuildInterval;
        for (int64_t k = 0; k < P && rc == MRMD_OK; k += K)
        {
            rc = step(ctx, b, st0 + k, false);
            if (rc == MRMD_OK && K > 1) rc = persistent_steps(ctx, b, (int)(K - 1));
        }
    }
    else
    {
        for (int64_t k = 0; k < P && rc == MRMD_OK; ++k) rc = step(ctx, b, st0 + k, false);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    b->graphKernels = ctx->launches - l0;
    ctx->launches = l0;
    b->rebuilds = r0;  // counted when the graph runs
    if (rc != MRMD_OK)
    {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    MRMD_TRY(check_cuda(ctx, e, "batch end capture"));
    b->graph = g;
    MRMD_CUDA(ctx, cudaGraphInstantiate(&b->exec, g, 0));
    return MRMD_OK;
}

// energies of steps [st0, st0 + count) from the ring into out[k][R]
int read_ring(mrmd_ctx* ctx, mrmd_batch* b, int64_t st0, int64_t count, double* out)
{
    if (!out || count <= 0) return MRMD_OK;
    const int64_t R = b->R, ring = b->B.ring;
    MRMD_CUDA(ctx, cudaMemcpyAsync(b->hRing, b->B.energyRing, sizeof(double) * (size_t)(ring * R),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t k = 0; k < count; ++k)
        std::memcpy(out + k * R, b->hRing + ((st0 + k) % ring) * R, sizeof(double) * (size_t)R);
    return MRMD_OK;
}

int run_graph(mrmd_ctx* ctx, mrmd_batch* b, int64_t st0)
{
    BDev& B = b->B;
    for (int attempt = 0;; ++attempt)
    {
        if (!b->exec) MRMD_TRY(capture(ctx, b, st0));
        MRMD_CUDA(ctx, cudaMemsetAsync(&B.sc->overflow, 0, sizeof(uint32_t), ctx->stream));
        MRMD_CUDA(ctx, cudaMemsetAsync(b->dSync + 2, 0, sizeof(unsigned), ctx->stream));
        MRMD_TRY(snapshot(ctx, b, b->sn, true));
        MRMD_CUDA(ctx, cudaGraphLaunch(b->exec, ctx->stream));
        ctx->launches += b->graphKernels;
        b->graphLaunches++;
        MRMD_CUDA(ctx, cudaMemcpyAsync(b->hSc, B.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, ctx->stream));
        unsigned syncError = 0;
        MRMD_CUDA(ctx, cudaMemcpyAsync(&syncError, b->dSync + 2, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (syncError)
            return set_error(ctx, MRMD_ERR_TIMEOUT, "a grid barrier of the persistent step kernel timed out");
        const uint32_t f = b->hSc->overflow;
        const int64_t P = b->cfg.tuning.graphSteps;
        if (!f)
        {
            b->rebuilds += P / b->cfg.tuning.rebuildInterval;
            return MRMD_OK;
        }
        if (attempt >= 4) return set_error(ctx, MRMD_ERR_NLIST_OVERFLOW, "batch buffers kept overflowing");
        // roll back, grow, re-capture
        const int32_t needG = b->hSc->numGhost, needL = b->hSc->maxCount, needF = b->hSc->maxCountF;
        const int32_t needC = b->hSc->maxCountC;
        MRMD_TRY(snapshot(ctx, b, b->sn, false));
        int32_t gCap = B.gCap, lCap = B.listCap, fCap = B.listCapF, cCap = B.listCapC;
        if (f & FLAG_GHOST_OVERFLOW) gCap = needG + needG / 4 + 1024;
        if (f & FLAG_LIST_OVERFLOW) lCap = needL + needL / 5 + 8;
        if (f & FLAG_FAR_LIST_OVERFLOW) fCap = needF + needF / 5 + 8;
        if (f & FLAG_CLUSTER_LIST_OVERFLOW) cCap = needC + needC / 5 + 8;
        MRMD_TRY(set_capacity(ctx, b, gCap, lCap, fCap, cCap));
        drop_graph(b);
        b->recoveries++;
    }
}

// the step decisions of the current device step (after creation, a restored
// state or a new ring size)
int refresh_step_flags(mrmd_ctx* ctx, mrmd_batch* b)
{
    MRMD_TRY(d2h(ctx, b->hSc, b->B.sc, sizeof(Scalars)));
    set_step_flags(*b->hSc, b->hSc->step, b->hSc->run, b->B.ring, b->B.compSampling, b->B.tfEnabled,
                   b->B.tfSampleInterval);
    return h2d(ctx, b->B.sc, b->hSc, sizeof(Scalars));
}

int validate_tuning(mrmd_ctx* ctx, const mrmd_batch_tuning& t)
{
    MRMD_CHECK_ARG(t.threadsPerRow == 1 || t.threadsPerRow == 2 || t.threadsPerRow == 4 || t.threadsPerRow == 8, ctx,
                   "threadsPerRow must be 1, 2, 4 or 8");
    MRMD_CHECK_ARG(t.blockSize >= 64 && t.blockSize <= 1024 && t.blockSize % 32 == 0, ctx, "bad blockSize");
    MRMD_CHECK_ARG(t.rebuildInterval >= 1 && t.sortEvery >= 0 && t.graphSteps >= 0, ctx, "bad tuning intervals");
    MRMD_CHECK_ARG(t.listLayout >= LAYOUT_ROWS && t.listLayout <= LAYOUT_CLUSTER, ctx, "listLayout must be 0, 1 or 2");
    MRMD_CHECK_ARG(t.listLayout != LAYOUT_CLUSTER || t.threadsPerRow == CLUSTER_J, ctx,
                   "the cluster layout (listLayout 2) takes threadsPerRow 4");
    MRMD_CHECK_ARG(t.persistent == 0 || t.persistent == 1, ctx, "persistent must be 0 or 1");
    const int64_t period = t.rebuildInterval * (t.sortEvery > 0 ? t.sortEvery : 1);
    MRMD_CHECK_ARG(t.graphSteps == 0 || t.graphSteps % period == 0, ctx,
                   "graphSteps must be a multiple of rebuildInterval * sortEvery");
    return MRMD_OK;
}

// ring size and pinned host copy follow graphSteps
int ensure_ring(mrmd_ctx* ctx, mrmd_batch* b)
{
    const int32_t need = (int32_t)std::max<int64_t>(b->cfg.tuning.graphSteps, 64);
    if (need <= b->B.ring) return MRMD_OK;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    dfree(b->B.energyRing);
    b->B.energyRing = nullptr;
    if (b->hRing) cudaFreeHost(b->hRing);
    b->hRing = nullptr;
    MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&b->B.energyRing), sizeof(double) * (size_t)need * b->R));
    MRMD_TRY(dzero(ctx, b->B.energyRing, sizeof(double) * (size_t)need * b->R));
    MRMD_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&b->hRing), sizeof(double) * (size_t)need * b->R));
    b->B.ring = need;
    drop_graph(b);
    return MRMD_OK;
}

void free_all(mrmd_batch* b)
{
    drop_graph(b);
    BDev& B = b->B;
    void* ptrs[] = {B.pos, B.vel, B.force, B.mass, B.orig, B.slotRep, B.gSrc, B.gShift, B.imgFlags, B.ref, B.xImg, B.gCount,
                    B.lam, B.lamt, B.lamtf, B.hi, B.lo, B.cellOf, B.cellStart, B.cursor, B.unordered, B.sorted,
                    B.spos, B.counts, B.nbrs, B.countsF, B.nbrsF, B.clusters, B.countsC, B.clist, B.sPos, B.sVel, B.sMass, B.sOrig, B.tfForce,
                    B.tfDensity, B.tfWork, B.compEnergy, B.compCounter, B.compMean, B.energyRing, B.sc,
                    b->dReps, b->dTfFF, b->dSync};
    for (void* p : ptrs) dfree(p);
    snap_free(b->sn);
    if (b->hSc) cudaFreeHost(b->hSc);
    if (b->hRing) cudaFreeHost(b->hRing);
}
}  // namespace mrmd_batch_impl

extern "C" {

int mrmd_batch_create(mrmd_ctx* ctx, mrmd_batch** out, const mrmd_batch_config* cfg, int64_t numReplicas,
                      const mrmd_replica_desc* replicas, const double* pos3, const double* vel3)
{
    if (!ctx || !out || !cfg || !replicas || !pos3 || !vel3 || numReplicas <= 0) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(cfg->rc > 0 && cfg->skin >= 0 && cfg->dt > 0, ctx, "bad config");
    MRMD_CHECK_ARG(cfg->precision == MRMD_PREC_FP64 || cfg->precision == MRMD_PREC_MIXED, ctx, "bad precision");
    MRMD_CHECK_ARG(cfg->hybridDiameter > 0.0 && cfg->nu >= 1, ctx, "bad hybrid region");
    MRMD_CHECK_ARG(!cfg->tfEnabled || (cfg->tfSampleInterval >= 1 && cfg->tfUpdateInterval >= 1 && cfg->tfBinWidth > 0),
                   ctx, "bad thermodynamic-force settings");
    MRMD_TRY(validate_tuning(ctx, cfg->tuning));
    *out = nullptr;
    mrmd_batch* b = new mrmd_batch();
    b->cfg = *cfg;
    if (b->cfg.compSamplingInterval <= 0) b->cfg.compSamplingInterval = 200;   // LJ_IdealGas.hpp:69
    if (b->cfg.compUpdateInterval <= 0) b->cfg.compUpdateInterval = 20000;    // LJ_IdealGas.hpp:70
    const double rlist = cfg->rc + cfg->skin;
    const double ghost3[3] = {rlist, rlist, rlist};
    b->R = (int32_t)numReplicas;
    b->offsets.assign((size_t)numReplicas + 1, 0);
    b->reps.resize((size_t)numReplicas);
    int rc = MRMD_OK;
    int64_t cellBase = 0, binBase = 0;
    for (int64_t r = 0; r < numReplicas && rc == MRMD_OK; ++r)
    {
        const mrmd_replica_desc& d = replicas[r];
        RepDev& R = b->reps[(size_t)r];
        mrmd_subdomain sd{};
        if (d.numMolecules < 1 || mrmd_subdomain_init(&sd, d.boxMin, d.boxMax, ghost3) != MRMD_OK)
        {
            rc = set_error(ctx, MRMD_ERR_ARG, "replica %lld: bad size or box", (long long)r);
            break;
        }
        for (int a = 0; a < 3; ++a)
            if (!(sd.diameter[a] > rlist)) rc = set_error(ctx, MRMD_ERR_ARG, "replica %lld: box must exceed the list radius", (long long)r);
        const CellGrid g = make_grid(sd.minGhostCorner, sd.maxGhostCorner, rlist);
        for (int a = 0; a < 3; ++a)
        {
            R.lo[a] = sd.minCorner[a];
            R.mx[a] = sd.maxCorner[a];
            R.L[a] = sd.diameter[a];
            R.minIn[a] = sd.minInnerCorner[a];
            R.maxIn[a] = sd.maxInnerCorner[a];
        }
        R.gmn[0] = g.mn.x;
        R.gmn[1] = g.mn.y;
        R.gmn[2] = g.mn.z;
        R.grdx[0] = g.rdx.x;
        R.grdx[1] = g.rdx.y;
        R.grdx[2] = g.rdx.z;
        R.gn[0] = g.n.x;
        R.gn[1] = g.n.y;
        R.gn[2] = g.n.z;
        R.cellBase = (int32_t)cellBase;
        cellBase += g.ncell;
        b->listExtent = std::fmax(b->listExtent, g.extent);
        double ext = 0.0;
        for (int a = 0; a < 3; ++a) ext = std::fmax(ext, sd.diameterWithGhostLayer[a]);
        const SplitParams sp = split_params(sd.minGhostCorner, ext * 1.25 + 8.0);
        R.splitScale = sp.scale;
        R.splitInv = sp.invScale;
        {
            int e = 0;
            std::frexp(sp.invScale, &e);  // 2^-q = 0.5 * 2^e
            R.sq = 1 - e;
        }
        for (int a = 0; a < 3; ++a)
        {
            // the split origin on the 2^-q grid (the pair kernels use only
            // differences of split coordinates), taken by split_bits as an
            // integer multiple of 2^-q
            const double o = std::floor(R.gmn[a] / sp.invScale) * sp.invScale;
            if (!(std::fabs(o) < sp.invScale * 1099511627776.0))
                rc = set_error(ctx, MRMD_ERR_ARG, "replica %lld too far from the origin for the mixed form",
                               (long long)r);
            R.sko[a] = (long long)(o / sp.invScale);
            R.soff[a] = (float)(R.gmn[a] - o);
        }
        mrmd_slab slab{};
        slab.center[0] = d.slabCenter[0];
        slab.center[1] = d.slabCenter[1];
        slab.center[2] = d.slabCenter[2];
        slab.atomisticRegionDiameter = d.atomisticDiameter;
        slab.hybridRegionDiameter = cfg->hybridDiameter;
        slab.nu = cfg->nu;
        slab.interfaceType = 0;
        R.slab = to_slab(&slab);
        // every molecule within r_list (+ skin of drift) of an x face and every
        // image lies outside the slab's outer edge on both sides
        const double rOut = R.slab.atHalf + R.slab.hy, margin = rlist + cfg->skin + 1e-9 * (1.0 + sd.diameter[0]);
        R.consistent = (R.slab.cx - rOut > sd.minCorner[0] + margin) && (R.slab.cx + rOut < sd.maxCorner[0] - margin);
        R.lbase = (int32_t)b->offsets[(size_t)r];
        R.n = (int32_t)d.numMolecules;
        b->offsets[(size_t)r + 1] = b->offsets[(size_t)r] + d.numMolecules;
        R.seed = d.seed;
        // ThermodynamicForce on x bins (ThermodynamicForce.cpp:25-57, MultiHistogram.hpp:40-41)
        R.tfBins = 0;
        if (cfg->tfEnabled)
        {
            const int64_t nb = (int64_t)std::ceil(sd.diameter[0] / cfg->tfBinWidth);
            R.tfBins = (int32_t)nb;
            R.tfMin = sd.minCorner[0];
            R.tfBinSize = (sd.maxCorner[0] - sd.minCorner[0]) / (double)nb;
            R.tfInvBin = 1.0 / R.tfBinSize;
            R.tfBinVolume = sd.diameter[1] * sd.diameter[2] * R.tfBinSize;
            if (!(R.tfBinSize <= cfg->tfBinWidth)) rc = set_error(ctx, MRMD_ERR_ARG, "requested bin size is not achieved");
        }
        R.tfBase = (int32_t)binBase;
        binBase += R.tfBins;
    }
    const int64_t N = b->offsets.back();
    if (rc == MRMD_OK && (N > INT32_MAX / 4 || cellBase > INT32_MAX - 1))
        rc = set_error(ctx, MRMD_ERR_CAPACITY, "too many molecules or cells");
    if (rc != MRMD_OK)
    {
        delete b;
        return rc;
    }
    b->N = (int32_t)N;
    b->totalCells = cellBase;
    b->totalBins = binBase;
    BDev& B = b->B;
    B.R = b->R;
    B.N = b->N;
    B.totalCells = cellBase;
    B.totalBins = binBase;
    // physics
    {
        mrmd_lj_params t{};
        const double c = cfg->cappingDistance, r = cfg->rc, sg = cfg->sigma, e = cfg->epsilon;
        lj_table_host(&t, 1, &c, &r, &sg, &e, cfg->shifted);
        B.lj = to_dev(t);
        B.rcSqr = cfg->rc * cfg->rc;  // LJ_IdealGas.cpp:290-291
        B.rc2 = make_rcsq(B.rcSqr);
    }
    B.dt = cfg->dt;
    B.dtHalfOverMass = 0.5 * cfg->dt / 1.0;  // molecules have unit mass (UpdateSteps.hpp:25-39 with m = 1)
    B.ouDamping = std::exp(-cfg->gamma * cfg->dt);
    B.ouSigma = std::sqrt(cfg->temperature * (1.0 - std::exp(-2.0 * cfg->gamma * cfg->dt)));
    B.zeta = cfg->gamma;
    B.temperature = cfg->temperature;
    B.rlist = rlist;
    B.halfSkin = 0.5 * cfg->skin;
    {
        const double rs = lj_split_radius(cfg->sigma, cfg->cappingDistance);
        B.rsplitSq = (float)(rs * rs);
        B.nearSqF = (float)((rs + 0.5 * cfg->skin) * (rs + 0.5 * cfg->skin));
    }
    B.cgMargin = cfg->skin + 1e-3;  // twice the skin/2 a molecule may move between rebuilds
    B.K = cfg->tuning.rebuildInterval;
    B.tfEnabled = cfg->tfEnabled;
    B.tfSampleInterval = cfg->tfEnabled ? cfg->tfSampleInterval : 1;
    B.tfUpdateInterval = cfg->tfEnabled ? cfg->tfUpdateInterval : 1;
    B.compSampling = cfg->compFrozen ? 0 : b->cfg.compSamplingInterval;
    B.compUpdate = cfg->compFrozen ? 0 : b->cfg.compUpdateInterval;
    B.tfSigma = cfg->tfSmoothingSigma;
    B.tfRange = cfg->tfSmoothingRange;
    {
        // FP32 error band of the list build (as in build_half_list)
        const double delta = std::ldexp(b->listExtent, -22);
        const double band = 6.0 * rlist * delta + 3.0 * delta * delta + std::ldexp(rlist * rlist, -20);
        B.listRsq = rlist * rlist;
        B.listRsqLo = (float)std::fmax(0.0, (B.listRsq - 2.0 * band) * (1.0 - 1e-6));
        B.listRsqHi = (float)((B.listRsq + 2.0 * band) * (1.0 + 1e-6));
    }
    // buffers
    const int64_t nb = std::max<int64_t>(binBase, 1), nc = (int64_t)b->R * COMP_BINS;
    auto alloc = [&](auto*& p, int64_t count) {
        if (rc == MRMD_OK) rc = grow(ctx, p, 0, count);
        if (rc == MRMD_OK) rc = dzero(ctx, p, sizeof(*p) * (size_t)std::max<int64_t>(count, 1));
    };
    alloc(B.vel, N);
    alloc(B.force, N);
    alloc(B.mass, N);
    alloc(B.orig, N);
    alloc(B.imgFlags, N);
    alloc(B.ref, N);
    alloc(B.xImg, N);
    alloc(B.gCount, N + 1);
    alloc(B.counts, N);
    alloc(B.countsF, N);
    alloc(B.sPos, N);
    alloc(B.sVel, N);
    alloc(B.sMass, N);
    alloc(B.sOrig, N);
    alloc(B.cellStart, cellBase + 1);
    alloc(B.cursor, cellBase + 1);
    alloc(B.tfForce, nb);
    alloc(B.tfDensity, nb);
    alloc(B.tfWork, 3 * nb);
    alloc(B.compEnergy, nc);
    alloc(B.compCounter, nc);
    alloc(B.compMean, nc);
    alloc(B.sc, 1);
    alloc(b->dSync, 4);
    alloc(b->dReps, b->R);
    alloc(b->dTfFF, 1);
    {
        // i-clusters of the cluster layout: CLUSTER_I molecules of one
        // replica, aligned to the replica's first molecule
        std::vector<int2> cls;
        for (int32_t r = 0; r < b->R; ++r)
            for (int64_t i = b->offsets[(size_t)r]; i < b->offsets[(size_t)r + 1]; i += CLUSTER_I)
                cls.push_back(make_int2((int32_t)i, (int32_t)std::min<int64_t>(CLUSTER_I, b->offsets[(size_t)r + 1] - i)));
        B.numClusters = (int32_t)cls.size();
        alloc(B.clusters, B.numClusters);
        alloc(B.countsC, B.numClusters);
        if (rc == MRMD_OK) rc = h2d(ctx, B.clusters, cls.data(), sizeof(int2) * cls.size());
    }
    if (rc == MRMD_OK) rc = snap_alloc(ctx, b, b->sn);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaMallocHost(reinterpret_cast<void**>(&b->hSc), sizeof(Scalars)), "batch pinned");
    if (rc == MRMD_OK) rc = ensure_ring(ctx, b);
    // initial guesses for the ghost and list capacity: measured below
    const int32_t g0 = cfg->initialGhostCapacity > 0 ? (int32_t)cfg->initialGhostCapacity : (int32_t)std::min<int64_t>(2 * N + 1024, INT32_MAX / 2);
    const int32_t l0 = cfg->initialMaxNeighbors > 0 ? (int32_t)cfg->initialMaxNeighbors : 64;
    const int32_t f0 = cfg->initialMaxNeighbors > 0 ? (int32_t)cfg->initialMaxNeighbors : 96;
    if (rc == MRMD_OK) rc = set_capacity(ctx, b, g0, l0, f0);
    if (rc == MRMD_OK) rc = apply_layout(ctx, b);
    B.reps = b->dReps;
    B.tfFF = b->dTfFF;
    if (rc == MRMD_OK)
        rc = h2d(ctx, b->dReps, b->reps.data(), sizeof(RepDev) * b->reps.size());
    if (rc == MRMD_OK)
    {
        const double ff = cfg->tfTargetDensity != 0.0 ? cfg->tfModulation / cfg->tfTargetDensity : 0.0;
        rc = h2d(ctx, b->dTfFF, &ff, sizeof(double));
    }
    if (rc == MRMD_OK)
    {
        // molecules, replica after replica (slot i = input index i)
        std::vector<double4> p4((size_t)N), v4((size_t)N);
        std::vector<int32_t> rep((size_t)N), orig((size_t)N);
        std::vector<double> mass((size_t)N, 1.0);
        for (int32_t r = 0; r < b->R; ++r)
            for (int64_t i = b->offsets[(size_t)r]; i < b->offsets[(size_t)r + 1]; ++i) rep[(size_t)i] = r;
        for (int64_t i = 0; i < N; ++i)
        {
            p4[(size_t)i] = make_double4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], 0.0);
            v4[(size_t)i] = make_double4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.0);
            orig[(size_t)i] = (int32_t)i;
        }
        rc = h2d(ctx, B.pos, p4.data(), sizeof(double4) * (size_t)N);
        if (rc == MRMD_OK) rc = h2d(ctx, B.vel, v4.data(), sizeof(double4) * (size_t)N);
        if (rc == MRMD_OK) rc = h2d(ctx, B.mass, mass.data(), sizeof(double) * (size_t)N);
        if (rc == MRMD_OK) rc = h2d(ctx, B.orig, orig.data(), sizeof(int32_t) * (size_t)N);
        if (rc == MRMD_OK) rc = h2d(ctx, B.slotRep, rep.data(), sizeof(int32_t) * (size_t)N);
    }
    if (rc == MRMD_OK)
    {
        // size the buffers on the initial configuration: a rebuild that only
        // writes ghosts, cells and lists (overwritten by the first step);
        // it also sizes the scan scratch before any graph capture
        const int oldSync = ctx->sync;
        ctx->sync = 0;
        rc = rebuild(ctx, b, false);
        // the context stream does not synchronise with the legacy stream
        if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "probe");
        if (rc == MRMD_OK) rc = d2h(ctx, b->hSc, B.sc, sizeof(Scalars));
        ctx->sync = oldSync;
        if (rc == MRMD_OK)
        {
            const int32_t ng = b->hSc->numGhost;
            int32_t mc = b->hSc->maxCount;
            if (!(b->hSc->overflow & FLAG_LIST_OVERFLOW))
            {
                // no overflow: the largest row is below the guess; measure it
                std::vector<int32_t> counts((size_t)N);
                rc = d2h(ctx, counts.data(), B.counts, sizeof(int32_t) * (size_t)N);
                mc = 0;
                for (int32_t c : counts) mc = std::max(mc, c);
            }
            int32_t mcF = b->hSc->maxCountF;
            if (rc == MRMD_OK && B.split && !(b->hSc->overflow & FLAG_FAR_LIST_OVERFLOW))
            {
                std::vector<int32_t> counts((size_t)N);
                rc = d2h(ctx, counts.data(), B.countsF, sizeof(int32_t) * (size_t)N);
                mcF = 0;
                for (int32_t c : counts) mcF = std::max(mcF, c);
            }
            const bool cluster = cfg->tuning.listLayout == LAYOUT_CLUSTER;
            int32_t mcC = b->hSc->maxCountC;
            if (rc == MRMD_OK && cluster && !(b->hSc->overflow & FLAG_CLUSTER_LIST_OVERFLOW))
            {
                std::vector<int32_t> counts((size_t)B.numClusters);
                rc = d2h(ctx, counts.data(), B.countsC, sizeof(int32_t) * counts.size());
                mcC = 0;
                for (int32_t c : counts) mcC = std::max(mcC, c);
            }
            const int32_t gCap = cfg->initialGhostCapacity > 0 ? (int32_t)cfg->initialGhostCapacity : ng + ng / 3 + 1024;
            const int32_t lCap = cfg->initialMaxNeighbors > 0 ? (int32_t)cfg->initialMaxNeighbors : mc + mc / 3 + 8;
            const int32_t fCap = B.split ? mcF + mcF / 3 + 8 : B.listCapF;
            const int32_t cCap = !cluster ? B.listCapC
                                 : cfg->initialMaxNeighbors > 0 ? (int32_t)cfg->initialMaxNeighbors
                                                                : mcC + mcC / 3 + 8;
            Scalars z{};
            if (rc == MRMD_OK) rc = h2d(ctx, B.sc, &z, sizeof(Scalars));
            if (rc == MRMD_OK) rc = set_capacity(ctx, b, gCap, lCap, fCap, cCap);
        }
    }
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaDeviceSynchronize(), "batch create");
    if (rc != MRMD_OK)
    {
        free_all(b);
        delete b;
        return rc;
    }
    *out = b;
    return MRMD_OK;
}

int mrmd_batch_destroy(mrmd_ctx* ctx, mrmd_batch* b)
{
    if (!b) return MRMD_OK;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    free_all(b);
    delete b;
    return MRMD_OK;
}

int mrmd_batch_run(mrmd_ctx* ctx, mrmd_batch* b, int64_t nsteps, double* energies)
{
    if (!ctx || !b || nsteps < 0) return MRMD_ERR_ARG;
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    const int64_t P = b->cfg.tuning.graphSteps;
    int rc = refresh_step_flags(ctx, b);
    int64_t k = 0;
    while (rc == MRMD_OK && k < nsteps)
    {
        const int64_t st = b->steps + k;
        if (P > 0 && st % P == 0 && nsteps - k >= P)
        {
            rc = run_graph(ctx, b, st);
            if (rc == MRMD_OK) rc = read_ring(ctx, b, st, P, energies ? energies + k * b->R : nullptr);
            k += P;
        }
        else
        {
            rc = step(ctx, b, st, true);
            if (rc == MRMD_OK) rc = read_ring(ctx, b, st, 1, energies ? energies + k * b->R : nullptr);
            ++k;
        }
    }
    b->steps += k;
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "batch run");
}

int mrmd_batch_get_state(mrmd_ctx* ctx, mrmd_batch* b, double* pos3, double* vel3, double* force3)
{
    if (!ctx || !b) return MRMD_ERR_ARG;
    const size_t N = (size_t)b->N;
    std::vector<double4> h(N);
    std::vector<int32_t> orig(N);
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MRMD_TRY(d2h(ctx, orig.data(), b->B.orig, sizeof(int32_t) * N));
    double* outs[3] = {pos3, vel3, force3};
    const double4* src[3] = {b->B.pos, b->B.vel, b->B.force};
    for (int q = 0; q < 3; ++q)
    {
        if (!outs[q]) continue;
        MRMD_TRY(d2h(ctx, h.data(), src[q], sizeof(double4) * N));
        for (size_t i = 0; i < N; ++i)
        {
            const size_t o = (size_t)orig[i];
            outs[q][3 * o] = h[i].x;
            outs[q][3 * o + 1] = h[i].y;
            outs[q][3 * o + 2] = h[i].z;
        }
    }
    return MRMD_OK;
}

int mrmd_batch_get_tf(mrmd_ctx* ctx, mrmd_batch* b, double* force, double* density, int64_t* binOffsets)
{
    if (!ctx || !b) return MRMD_ERR_ARG;
    const size_t nb = (size_t)b->totalBins;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (force && nb) MRMD_TRY(d2h(ctx, force, b->B.tfForce, sizeof(double) * nb));
    if (density && nb)
    {
        std::vector<unsigned long long> c(nb);
        MRMD_TRY(d2h(ctx, c.data(), b->B.tfDensity, sizeof(unsigned long long) * nb));
        for (size_t k = 0; k < nb; ++k) density[k] = (double)c[k];
    }
    if (binOffsets)
    {
        for (int32_t r = 0; r < b->R; ++r) binOffsets[r] = b->reps[(size_t)r].tfBase;
        binOffsets[b->R] = b->totalBins;
    }
    return MRMD_OK;
}

int mrmd_batch_set_tf(mrmd_ctx* ctx, mrmd_batch* b, const double* force)
{
    if (!ctx || !b || !force) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (b->totalBins)
        MRMD_TRY(h2d(ctx, b->B.tfForce, force, sizeof(double) * (size_t)b->totalBins));
    return MRMD_OK;
}

int mrmd_batch_get_compensation(mrmd_ctx* ctx, mrmd_batch* b, double* mean)
{
    if (!ctx || !b || !mean) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MRMD_TRY(d2h(ctx, mean, b->B.compMean, sizeof(double) * (size_t)b->R * COMP_BINS));
    return MRMD_OK;
}

int mrmd_batch_set_compensation(mrmd_ctx* ctx, mrmd_batch* b, const double* mean)
{
    if (!ctx || !b || !mean) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return h2d(ctx, b->B.compMean, mean, sizeof(double) * (size_t)b->R * COMP_BINS);
}

int mrmd_batch_get_tuning(const mrmd_batch* b, mrmd_batch_tuning* t)
{
    if (!b || !t) return MRMD_ERR_ARG;
    *t = b->cfg.tuning;
    return MRMD_OK;
}

int mrmd_batch_set_tuning(mrmd_ctx* ctx, mrmd_batch* b, const mrmd_batch_tuning* t)
{
    if (!ctx || !b || !t) return MRMD_ERR_ARG;
    MRMD_TRY(validate_tuning(ctx, *t));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    b->cfg.tuning = *t;
    MRMD_TRY(apply_layout(ctx, b));
    b->B.K = t->rebuildInterval;
    b->needRebuild = true;
    drop_graph(b);
    return ensure_ring(ctx, b);
}

int mrmd_batch_list_stats(mrmd_ctx* ctx, mrmd_batch* b, int64_t* out3)
{
    if (!ctx || !b || !out3) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (b->cfg.tuning.listLayout == LAYOUT_CLUSTER)
    {
        unsigned long long* d = nullptr;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&d), 2 * sizeof(unsigned long long)));
        unsigned long long h[2] = {0, 0};
        int rc = check_cuda(ctx, cudaMemsetAsync(d, 0, sizeof(h), ctx->stream), "memset");
        if (rc == MRMD_OK)
        {
            k_b_cluster_stats<<<grid_for(ctx, b->B.numClusters, TB), TB, 0, ctx->stream>>>(b->B, d);
            rc = after_launch(ctx, "batch cluster_stats");
        }
        if (rc == MRMD_OK) rc = d2h(ctx, h, d, sizeof(h));
        dfree(d);
        MRMD_TRY(rc);
        out3[0] = (int64_t)h[0];
        out3[1] = (int64_t)h[1];
        out3[2] = 32;
        return MRMD_OK;
    }
    std::vector<int32_t> counts((size_t)b->N);
    MRMD_TRY(d2h(ctx, counts.data(), b->B.counts, sizeof(int32_t) * counts.size()));
    int64_t pairs = 0;
    for (int32_t c : counts) pairs += c;
    if (b->B.split)
    {
        MRMD_TRY(d2h(ctx, counts.data(), b->B.countsF, sizeof(int32_t) * counts.size()));
        for (int32_t c : counts) pairs += c;
    }
    out3[0] = pairs;
    out3[1] = pairs;
    out3[2] = 1;
    return MRMD_OK;
}

int mrmd_grid_sync_selftest(mrmd_ctx* ctx, int32_t rounds, int32_t skipBlock, double limitMs)
{
    if (!ctx || rounds < 0 || !(limitMs > 0.0)) return MRMD_ERR_ARG;
    unsigned* d = nullptr;
    MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&d), 4 * sizeof(unsigned)));
    int rc = check_cuda(ctx, cudaMemsetAsync(d, 0, 4 * sizeof(unsigned), ctx->stream), "memset");
    const GridBar gb{d, d + 1, reinterpret_cast<int32_t*>(d + 2), (unsigned long long)(limitMs * 1e6)};
    if (rc == MRMD_OK)
        rc = cooperative_launch(ctx, k_grid_sync_test, 128, "grid sync selftest", gb, (int)rounds, (int)skipBlock);
    unsigned err = 0;
    if (rc == MRMD_OK) rc = d2h(ctx, &err, d + 2, sizeof(unsigned));
    cudaStreamSynchronize(ctx->stream);
    dfree(d);
    MRMD_TRY(rc);
    return err ? set_error(ctx, MRMD_ERR_TIMEOUT, "grid barrier wait gave up after %.1f ms", limitMs) : MRMD_OK;
}

int mrmd_batch_pair_keys(mrmd_ctx* ctx, mrmd_batch* b, int64_t replica, int64_t* keys, int64_t cap,
                         int64_t* count)
{
    if (!ctx || !b || !count || replica < 0 || replica >= b->R) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const BDev& B = b->B;
    const int64_t N = b->N;
    MRMD_TRY(d2h(ctx, b->hSc, B.sc, sizeof(Scalars)));
    const int64_t nGhost = b->hSc->numGhost;
    if (nGhost < 0 || nGhost > B.gCap) return set_error(ctx, MRMD_ERR_STATE, "ghost count outside the capacity");
    std::vector<int32_t> orig((size_t)N), slotRep((size_t)N), gSrc((size_t)std::max<int64_t>(nGhost, 1));
    MRMD_TRY(d2h(ctx, orig.data(), B.orig, sizeof(int32_t) * (size_t)N));
    MRMD_TRY(d2h(ctx, slotRep.data(), B.slotRep, sizeof(int32_t) * (size_t)N));
    if (nGhost > 0) MRMD_TRY(d2h(ctx, gSrc.data(), B.gSrc, sizeof(int32_t) * (size_t)nGhost));
    const int64_t off = b->offsets[(size_t)replica];
    std::vector<int64_t> out;
    bool bad = false;
    // slot j (a ghost maps to its source) -> key of the unordered pair with local i
    auto add = [&](int64_t i, int64_t j) {
        if (j >= N) j = j - N < nGhost ? gSrc[(size_t)(j - N)] : -1;
        if (j < 0 || j >= N)
        {
            bad = true;
            return;
        }
        const int64_t a = orig[(size_t)i] - off, c = orig[(size_t)j] - off;
        out.push_back(std::min(a, c) * (int64_t(1) << 32) + std::max(a, c));
    };
    if (b->cfg.tuning.listLayout == LAYOUT_CLUSTER)
    {
        const int64_t nc = B.numClusters, capC = B.listCapC;
        std::vector<int2> cl((size_t)std::max<int64_t>(nc, 1));
        std::vector<int32_t> cnt((size_t)std::max<int64_t>(nc, 1));
        std::vector<int4> cli((size_t)std::max<int64_t>(nc * capC, 1));
        std::vector<float4> sp((size_t)(N + nGhost));
        MRMD_TRY(d2h(ctx, cl.data(), B.clusters, sizeof(int2) * (size_t)nc));
        MRMD_TRY(d2h(ctx, cnt.data(), B.countsC, sizeof(int32_t) * (size_t)nc));
        MRMD_TRY(d2h(ctx, cli.data(), B.clist, sizeof(int4) * (size_t)(nc * capC)));
        MRMD_TRY(d2h(ctx, sp.data(), B.spos, sizeof(float4) * sp.size()));
        for (int64_t c = 0; c < nc; ++c)
        {
            if (cl[(size_t)c].x < 0 || cl[(size_t)c].x >= N || slotRep[(size_t)cl[(size_t)c].x] != replica) continue;
            for (int32_t e = 0; e < cnt[(size_t)c]; ++e)
            {
                const int4 v = cli[(size_t)(c * capC + e)];
                for (int bit = 0; bit < 32; ++bit)
                {
                    if (!(((uint32_t)v.y >> bit) & 1u)) continue;
                    const int64_t i = cl[(size_t)c].x + (bit >> 2), s = (int64_t)v.x + (bit & (CLUSTER_J - 1));
                    if (i >= N || s < 0 || s >= N + nGhost)
                    {
                        bad = true;
                        continue;
                    }
                    int32_t j;
                    std::memcpy(&j, &sp[(size_t)s].w, sizeof(j));
                    add(i, j);
                }
            }
        }
    }
    else
    {
        const int64_t tiles = div_up(N, 32);
        for (int w = 0; w < (B.split ? 2 : 1); ++w)
        {
            const int64_t lc = w == 0 ? B.listCap : B.listCapF;
            std::vector<int32_t> cnt((size_t)N), nb((size_t)std::max<int64_t>(tiles * 32 * lc, 1));
            MRMD_TRY(d2h(ctx, cnt.data(), w == 0 ? B.counts : B.countsF, sizeof(int32_t) * (size_t)N));
            MRMD_TRY(d2h(ctx, nb.data(), w == 0 ? B.nbrs : B.nbrsF, sizeof(int32_t) * (size_t)(tiles * 32 * lc)));
            for (int64_t i = 0; i < N; ++i)
            {
                if (slotRep[(size_t)i] != replica) continue;
                for (int64_t k = 0; k < cnt[(size_t)i] && k < lc; ++k)
                    add(i, nb[(size_t)((i >> 5) * (lc << 5) + (k << 5) + (i & 31))] & 0x7fffffff);
            }
        }
    }
    if (bad) return set_error(ctx, MRMD_ERR_STATE, "list entry outside the locals and ghosts");
    std::sort(out.begin(), out.end());
    *count = (int64_t)out.size();
    if (!keys) return MRMD_OK;
    if (cap < (int64_t)out.size()) return set_error(ctx, MRMD_ERR_CAPACITY, "pair key capacity %lld < %lld",
                                                     (long long)cap, (long long)out.size());
    std::copy(out.begin(), out.end(), keys);
    return MRMD_OK;
}

int mrmd_batch_stats(mrmd_ctx* ctx, mrmd_batch* b, int64_t* out10)
{
    if (!ctx || !b || !out10) return MRMD_ERR_ARG;
    int64_t ls[3];
    MRMD_TRY(mrmd_batch_list_stats(ctx, b, ls));
    MRMD_TRY(d2h(ctx, b->hSc, b->B.sc, sizeof(Scalars)));
    const int64_t pairs = ls[0];
    out10[0] = b->steps;
    out10[1] = b->rebuilds;
    out10[2] = pairs;
    out10[3] = b->hSc->numGhost;
    out10[4] = b->graphLaunches;
    out10[5] = ctx->launches;
    out10[6] = b->recoveries;
    out10[7] = b->cfg.tuning.listLayout == LAYOUT_CLUSTER ? b->B.listCapC
                                                          : b->B.listCap + (b->B.split ? b->B.listCapF : 0);
    out10[8] = b->B.gCap;
    out10[9] = b->hSc->flags | b->hSc->overflow;
    return MRMD_OK;
}

}  // extern "C"

namespace
{
// steps [b->steps, b->steps + n) through the same path as mrmd_batch_run,
// without energies
int advance(mrmd_ctx* ctx, mrmd_batch* b, int64_t n)
{
    MRMD_TRY(refresh_step_flags(ctx, b));
    const int64_t P = b->cfg.tuning.graphSteps;
    int64_t k = 0;
    while (k < n)
    {
        const int64_t st = b->steps + k;
        if (P > 0 && st % P == 0 && n - k >= P)
        {
            MRMD_TRY(run_graph(ctx, b, st));
            k += P;
        }
        else
        {
            MRMD_TRY(step(ctx, b, st, true));
            ++k;
        }
    }
    b->steps += k;
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_batch_autotune(mrmd_ctx* ctx, mrmd_batch* b, int64_t trialSteps, mrmd_batch_tuning* best,
                        double* msPerStep, mrmd_batch_tuning* candidates, int64_t* numCandidates)
{
    if (!ctx || !b || trialSteps < 1) return MRMD_ERR_ARG;
    const mrmd_batch_tuning t0 = b->cfg.tuning;
    // candidates: list layout x lanes per row x block size x rebuild interval;
    // the near/far rows exist in the mixed form only, the cluster layout has
    // CLUSTER_J lanes per row
    std::vector<mrmd_batch_tuning> cand;
    const int tprs[4] = {1, 2, 4, 8};
    const int blocks[3] = {64, 128, 256};
    const int64_t Ks[2] = {t0.rebuildInterval, 2 * t0.rebuildInterval};
    std::vector<int32_t> layouts{LAYOUT_ROWS};
    if (b->cfg.precision == MRMD_PREC_MIXED) layouts.push_back(LAYOUT_NEAR_FAR);
    layouts.push_back(LAYOUT_CLUSTER);
    for (int32_t layout : layouts)
        for (int64_t K : Ks)
            for (int tpr : tprs)
                for (int bs : blocks)
                {
                    if (layout == LAYOUT_CLUSTER && tpr != CLUSTER_J) continue;
                    mrmd_batch_tuning t = t0;
                    t.threadsPerRow = tpr;
                    t.blockSize = bs;
                    t.rebuildInterval = K;
                    t.listLayout = layout;
                    const int64_t period = K * (t.sortEvery > 0 ? t.sortEvery : 1);
                    if (t.graphSteps > 0) t.graphSteps = ((t0.graphSteps + period - 1) / period) * period;
                    cand.push_back(t);
                }
    // last candidate: the best of the others with the persistent step kernel
    // (filled in after they ran)
    if (t0.graphSteps > 0) cand.push_back(t0);
    const size_t numRegular = t0.graphSteps > 0 ? cand.size() - 1 : cand.size();
    const int oldSync = ctx->sync;
    ctx->sync = 0;
    Snap keep;
    int rc = snap_alloc(ctx, b, keep);
    if (rc == MRMD_OK) rc = snapshot(ctx, b, keep, true);
    const int64_t steps0 = b->steps, reb0 = b->rebuilds, gl0 = b->graphLaunches, rec0 = b->recoveries;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaEventCreate(&e0), "event");
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaEventCreate(&e1), "event");
    std::vector<double> ms(cand.size(), -1.0);
    int bestIdx = -1;
    for (size_t c = 0; c < cand.size() && rc == MRMD_OK; ++c)
    {
        if (c == numRegular)
        {
            if (bestIdx < 0) break;
            cand[c] = cand[(size_t)bestIdx];
            cand[c].persistent = 1;
        }
        b->cfg.tuning = cand[c];
        rc = apply_layout(ctx, b);
        if (rc != MRMD_OK) break;
        b->B.K = cand[c].rebuildInterval;
        b->needRebuild = true;
        drop_graph(b);
        rc = ensure_ring(ctx, b);
        // warm-up (captures the graph), then the timed trial from the same state
        if (rc == MRMD_OK) rc = advance(ctx, b, std::max<int64_t>(cand[c].graphSteps, 1));
        b->steps = steps0;
        b->needRebuild = true;
        if (rc == MRMD_OK) rc = snapshot(ctx, b, keep, false);
        if (rc == MRMD_OK) rc = check_cuda(ctx, cudaEventRecord(e0, ctx->stream), "event");
        if (rc == MRMD_OK) rc = advance(ctx, b, trialSteps);
        if (rc == MRMD_OK) rc = check_cuda(ctx, cudaEventRecord(e1, ctx->stream), "event");
        if (rc == MRMD_OK) rc = check_cuda(ctx, cudaEventSynchronize(e1), "event");
        float t = 0.0f;
        if (rc == MRMD_OK) rc = check_cuda(ctx, cudaEventElapsedTime(&t, e0, e1), "event");
        if (rc == MRMD_OK) rc = d2h(ctx, b->hSc, b->B.sc, sizeof(Scalars));
        if (rc == MRMD_OK)
        {
            // a longer rebuild interval than the configured one must keep every
            // molecule within skin/2 of its position at the last rebuild
            const bool safe = !(b->hSc->flags & FLAG_UNSAFE_INTERVAL) || cand[c].rebuildInterval <= t0.rebuildInterval;
            ms[c] = safe ? (double)t / (double)trialSteps : -1.0;
            if (safe && (bestIdx < 0 || ms[c] < ms[(size_t)bestIdx])) bestIdx = (int)c;
        }
        b->steps = steps0;
        if (rc == MRMD_OK) rc = snapshot(ctx, b, keep, false);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    b->rebuilds = reb0;
    b->graphLaunches = gl0;
    b->recoveries = rec0;
    b->cfg.tuning = bestIdx >= 0 ? cand[(size_t)bestIdx] : t0;
    if (rc == MRMD_OK) rc = apply_layout(ctx, b);
    b->B.K = b->cfg.tuning.rebuildInterval;
    b->needRebuild = true;
    drop_graph(b);
    if (rc == MRMD_OK) rc = ensure_ring(ctx, b);
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "autotune");
    snap_free(keep);
    ctx->sync = oldSync;
    MRMD_TRY(rc);
    if (best) *best = b->cfg.tuning;
    if (numCandidates) *numCandidates = (int64_t)cand.size();
    for (size_t c = 0; c < cand.size(); ++c)
    {
        if (msPerStep) msPerStep[c] = ms[c];
        if (candidates) candidates[c] = cand[c];
    }
    return bestIdx >= 0 ? MRMD_OK : set_error(ctx, MRMD_ERR_STATE, "no candidate kept the displacement below skin/2");
}

}  // extern "C"
