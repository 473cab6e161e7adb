// Periodic ghost layer: communication::GhostLayer and MultiResGhostLayer.
//
// Ghost creation follows GhostExchange::createGhostAtoms exactly: per axis
// X, Y, Z, every atom (real or earlier ghost) with x < minInner gets an
// image at +L and every atom with x >= maxInner one at -L; images of one
// pass are appended "+L images in source order, then -L images in source
// order".  A stable exclusive scan gives the same order as the reference's
// parallel_scan, so ghost indices are identical to the reference's.
#include "common.cuh"
#include "ghost_impl.cuh"

using namespace mrmd_impl;

namespace
{
constexpr int TB = 256;

__global__ void k_map_into_domain(double4* __restrict__ pos, int64_t n, double3 mn, double3 mx,
                                  double3 L)
{
    // communication/PeriodicMapping.cpp:30-58
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        double4 p = pos[i];
        double* c[3] = {&p.x, &p.y, &p.z};
        const double mnv[3] = {mn.x, mn.y, mn.z}, mxv[3] = {mx.x, mx.y, mx.z}, Lv[3] = {L.x, L.y, L.z};
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            double x = *c[d];
            if (mxv[d] <= x)
            {
                x = __dsub_rn(x, Lv[d]);
                x = fmax(x, mnv[d]);
            }
            if (x < mnv[d])
            {
                x = __dadd_rn(x, Lv[d]);
                if (mxv[d] <= x) x = mnv[d];
            }
            *c[d] = x;
        }
        pos[i] = p;
    }
}

__device__ __forceinline__ double comp(const double4& p, int axis)
{
    return axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
}

__device__ __forceinline__ void add_comp(double4& p, int axis, double v)
{
    if (axis == 0)
        p.x = __dadd_rn(p.x, v);
    else if (axis == 1)
        p.y = __dadd_rn(p.y, v);
    else
        p.z = __dadd_rn(p.z, v);
}

// packed (lo, hi) selection flags of one axis pass
__global__ void k_ghost_flags(const double4* __restrict__ pos, int64_t n, int axis, double minInner,
                              double maxInner, int64_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double x = comp(pos[i], axis);
        int64_t f = 0;
        if (x < minInner) f |= 1;
        if (x >= maxInner) f |= (int64_t)1 << 32;
        flags[i] = f;
    }
}

__device__ __forceinline__ void copy_atom(mrmd_atoms a, int64_t dst, int64_t src)
{
    // data/Atoms.hpp:97-110
    reinterpret_cast<double4*>(a.pos)[dst] = reinterpret_cast<const double4*>(a.pos)[src];
    reinterpret_cast<double4*>(a.vel)[dst] = reinterpret_cast<const double4*>(a.vel)[src];
    reinterpret_cast<double4*>(a.force)[dst] = reinterpret_cast<const double4*>(a.force)[src];
    a.type[dst] = a.type[src];
    a.mass[dst] = a.mass[src];
    a.charge[dst] = a.charge[src];
    a.relativeMass[dst] = a.relativeMass[src];
}

__global__ void k_ghost_copy(mrmd_atoms a, int32_t* __restrict__ corr, int64_t n, int axis,
                             double minInner, double maxInner, double L,
                             const int64_t* __restrict__ offsets, const int64_t* __restrict__ total)
{
    const int64_t numLo = (*total) & 0xffffffffLL;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double x = comp(reinterpret_cast<const double4*>(a.pos)[i], axis);
        const int64_t off = offsets[i];
        const int32_t real = corr[i] == -1 ? (int32_t)i : corr[i];
        if (x < minInner && MRMD_IN_BOUNDS(n + (off & 0xffffffffLL), a.capacity))
        {
            const int64_t dst = n + (off & 0xffffffffLL);
            copy_atom(a, dst, i);
            double4 p = reinterpret_cast<double4*>(a.pos)[dst];
            add_comp(p, axis, L);
            reinterpret_cast<double4*>(a.pos)[dst] = p;
            corr[dst] = real;
        }
        if (x >= maxInner && MRMD_IN_BOUNDS(n + numLo + (off >> 32), a.capacity))
        {
            const int64_t dst = n + numLo + (off >> 32);
            copy_atom(a, dst, i);
            double4 p = reinterpret_cast<double4*>(a.pos)[dst];
            add_comp(p, axis, -L);
            reinterpret_cast<double4*>(a.pos)[dst] = p;
            corr[dst] = real;
        }
    }
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// real -> ghosts CSR: count, scan, scatter, then sort each (tiny) segment
__global__ void k_csr_count(const int32_t* __restrict__ corr, int64_t nLocal, int64_t nGhost,
                            int32_t* __restrict__ cnt)
{
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nGhost;
         g += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t r = corr[nLocal + g];
        if (MRMD_IN_BOUNDS(r, nLocal)) atomicAdd(&cnt[r], 1);
    }
}

__global__ void k_csr_fill(const int32_t* __restrict__ corr, int64_t nLocal, int64_t nGhost,
                           const int32_t* __restrict__ start, int32_t* __restrict__ cursor,
                           int32_t* __restrict__ list)
{
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nGhost;
         g += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t r = corr[nLocal + g];
        if (!MRMD_IN_BOUNDS(r, nLocal)) continue;
        const int32_t k = atomicAdd(&cursor[r], 1);
        if (MRMD_IN_BOUNDS(start[r] + k, nGhost)) list[start[r] + k] = (int32_t)(nLocal + g);
    }
}

__global__ void k_csr_sort(const int32_t* __restrict__ start, int64_t nLocal, int32_t* __restrict__ list)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nLocal;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t s = start[i], e = start[i + 1];
        for (int32_t a = s + 1; a < e; ++a)
        {
            int32_t v = list[a];
            int32_t b = a - 1;
            while (b >= s && list[b] > v)
            {
                list[b + 1] = list[b];
                --b;
            }
            list[b + 1] = v;
        }
    }
}

__global__ void k_ghost_update(double4* __restrict__ pos, const int32_t* __restrict__ corr,
                               int64_t nLocal, int64_t nGhost, double3 L, double3 delta)
{
    // communication/UpdateGhostAtoms.cpp:31-68
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < nGhost;
         g += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t idx = nLocal + g;
        if (!MRMD_IN_BOUNDS(corr[idx], nLocal)) continue;
        pos[idx] = ghost_position(pos[idx], pos[corr[idx]], L, delta);
    }
}

__global__ void k_ghost_reduce(double4* __restrict__ force, const int32_t* __restrict__ start,
                               const int32_t* __restrict__ list, int64_t nLocal, int64_t nGhost)
{
    // communication/AccumulateForce.cpp:25-47, gathered per real atom in
    // ascending ghost order (the serial order of the reference loop)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nLocal;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t s = start[i], e = start[i + 1];
        if (s == e) continue;
        double4 f = force[i];
        for (int32_t k = s; k < e; ++k)
        {
            const int32_t g = list[k];
            if (!MRMD_IN_BOUNDS(g - nLocal, nGhost)) continue;
            const double4 fg = force[g];
            f.x = __dadd_rn(f.x, fg.x);
            f.y = __dadd_rn(f.y, fg.y);
            f.z = __dadd_rn(f.z, fg.z);
            force[g] = make_double4(0.0, 0.0, 0.0, 0.0);
        }
        force[i] = f;
    }
}

// ------------------------------------------------------- multi-resolution --

__global__ void k_multires_map(mrmd_molecules m, double4* __restrict__ apos, int64_t nMol,
                               double3 mn, double3 mx, double3 L)
{
    // communication/MultiResRealAtomsExchange.cpp:23-73
    for (int64_t mi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; mi < nMol;
         mi += (int64_t)gridDim.x * blockDim.x)
    {
        double4 p = reinterpret_cast<double4*>(m.pos)[mi];
        const int64_t s = m.atomsOffset[mi], e = s + m.numAtoms[mi];
        const double mnv[3] = {mn.x, mn.y, mn.z}, mxv[3] = {mx.x, mx.y, mx.z}, Lv[3] = {L.x, L.y, L.z};
        for (int d = 0; d < 3; ++d)
        {
            double x = comp(p, d);
            if (mxv[d] <= x)
            {
                x = __dsub_rn(x, Lv[d]);
                for (int64_t a = s; a < e; ++a)
                {
                    double4 q = apos[a];
                    add_comp(q, d, -Lv[d]);
                    apos[a] = q;
                }
            }
            if (x < mnv[d])
            {
                x = __dadd_rn(x, Lv[d]);
                for (int64_t a = s; a < e; ++a)
                {
                    double4 q = apos[a];
                    add_comp(q, d, Lv[d]);
                    apos[a] = q;
                }
            }
            if (d == 0) p.x = x;
            else if (d == 1) p.y = x;
            else p.z = x;
        }
        reinterpret_cast<double4*>(m.pos)[mi] = p;
    }
}

// two packed scans: hi = (x >= maxInner: molecules | atoms << 32), lo = (x < minInner)
__global__ void k_multires_flags(mrmd_molecules m, int64_t nMol, int axis, double minInner,
                                 double maxInner, int64_t* __restrict__ hi, int64_t* __restrict__ lo)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nMol;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double x = comp(reinterpret_cast<const double4*>(m.pos)[i], axis);
        const int64_t na = m.numAtoms[i];
        hi[i] = (x >= maxInner) ? (1 | (na << 32)) : 0;
        lo[i] = (x < minInner) ? (1 | (na << 32)) : 0;
    }
}

__device__ __forceinline__ void copy_molecule(mrmd_molecules m, int64_t dst, int64_t src)
{
    // data/Molecules.hpp:97-110
    reinterpret_cast<double4*>(m.pos)[dst] = reinterpret_cast<const double4*>(m.pos)[src];
    reinterpret_cast<double4*>(m.force)[dst] = reinterpret_cast<const double4*>(m.force)[src];
    reinterpret_cast<double4*>(m.gradLambda)[dst] = reinterpret_cast<const double4*>(m.gradLambda)[src];
    m.lambda[dst] = m.lambda[src];
    m.modulatedLambda[dst] = m.modulatedLambda[src];
    m.atomsOffset[dst] = m.atomsOffset[src];
    m.numAtoms[dst] = m.numAtoms[src];
}

__global__ void k_multires_copy(mrmd_molecules m, mrmd_atoms a, int32_t* __restrict__ corr,
                                int64_t nMol, int64_t nAtoms, int axis, double minInner,
                                double maxInner, double L, const int64_t* __restrict__ hiOff,
                                const int64_t* __restrict__ loOff, const int64_t* __restrict__ totals)
{
    // communication/MultiResPeriodicGhostExchange.cpp:147-240: "positive"
    // items (x >= maxInner, shifted by -L) first, then "negative" ones.
    const int64_t posM = totals[0] & 0xffffffffLL, posA = totals[0] >> 32;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nMol;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double x = comp(reinterpret_cast<const double4*>(m.pos)[i], axis);
        const int64_t s = m.atomsOffset[i], size = m.numAtoms[i];
        for (int side = 0; side < 2; ++side)
        {
            int64_t dstM, dstA;
            double shift;
            if (side == 0)
            {
                if (!(x >= maxInner)) continue;
                dstM = nMol + (hiOff[i] & 0xffffffffLL);
                dstA = nAtoms + (hiOff[i] >> 32);
                shift = -L;
            }
            else
            {
                if (!(x < minInner)) continue;
                dstM = nMol + posM + (loOff[i] & 0xffffffffLL);
                dstA = nAtoms + posA + (loOff[i] >> 32);
                shift = L;
            }
            copy_molecule(m, dstM, i);
            double4 p = reinterpret_cast<double4*>(m.pos)[dstM];
            add_comp(p, axis, shift);
            reinterpret_cast<double4*>(m.pos)[dstM] = p;
            m.atomsOffset[dstM] = dstA;
            m.numAtoms[dstM] = size;
            for (int64_t k = 0; k < size; ++k)
            {
                copy_atom(a, dstA + k, s + k);
                double4 q = reinterpret_cast<double4*>(a.pos)[dstA + k];
                add_comp(q, axis, shift);
                reinterpret_cast<double4*>(a.pos)[dstA + k] = q;
                const int32_t src = (int32_t)(s + k);
                corr[dstA + k] = corr[src] == -1 ? src : corr[src];
            }
        }
    }
}

int ensure_layer(mrmd_ctx* ctx, mrmd_ghost_layer* g, int64_t capacity, int64_t localCapacity)
{
    if (capacity > g->capacity)
    {
        int32_t* nc = nullptr;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&nc), sizeof(int32_t) * (size_t)capacity));
        if (g->correspondingRealAtom && g->capacity > 0)
            MRMD_CUDA(ctx, cudaMemcpyAsync(nc, g->correspondingRealAtom, sizeof(int32_t) * (size_t)g->capacity,
                                           cudaMemcpyDeviceToDevice, ctx->stream));
        int32_t* nl = nullptr;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&nl), sizeof(int32_t) * (size_t)capacity));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dfree(g->correspondingRealAtom);
        dfree(g->ghostList);
        g->correspondingRealAtom = nc;
        g->ghostList = nl;
        g->capacity = capacity;
    }
    if (localCapacity > g->localCapacity)
    {
        dfree(g->ghostStart);
        g->ghostStart = nullptr;
        MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&g->ghostStart), sizeof(int32_t) * (size_t)(localCapacity + 1)));
        g->localCapacity = localCapacity;
    }
    return MRMD_OK;
}

int build_csr(mrmd_ctx* ctx, mrmd_ghost_layer* g, int64_t nLocal, int64_t nGhost)
{
    int32_t* cursor = static_cast<int32_t*>(scratch(ctx, sizeof(int32_t) * (size_t)(nLocal + 1)));
    if (!cursor) return MRMD_ERR_OOM;
    MRMD_CUDA(ctx, cudaMemsetAsync(g->ghostStart, 0, sizeof(int32_t) * (size_t)(nLocal + 1), ctx->stream));
    if (nGhost > 0)
    {
        k_csr_count<<<grid_for(ctx, nGhost, TB), TB, 0, ctx->stream>>>(g->correspondingRealAtom, nLocal,
                                                                        nGhost, g->ghostStart);
        MRMD_TRY(after_launch(ctx, "csr_count"));
    }
    MRMD_TRY(scan_exclusive_i32(ctx, g->ghostStart, g->ghostStart, nLocal + 1, nullptr));
    if (nGhost > 0)
    {
        MRMD_CUDA(ctx, cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)(nLocal + 1), ctx->stream));
        k_csr_fill<<<grid_for(ctx, nGhost, TB), TB, 0, ctx->stream>>>(
            g->correspondingRealAtom, nLocal, nGhost, g->ghostStart, cursor, g->ghostList);
        MRMD_TRY(after_launch(ctx, "csr_fill"));
        k_csr_sort<<<grid_for(ctx, nLocal, TB), TB, 0, ctx->stream>>>(g->ghostStart, nLocal, g->ghostList);
        MRMD_TRY(after_launch(ctx, "csr_sort"));
    }
    return MRMD_OK;
}

inline double3 d3(const double* v) { return make_double3(v[0], v[1], v[2]); }
}  // namespace

extern "C" {

int mrmd_ghost_layer_alloc(mrmd_ctx* ctx, mrmd_ghost_layer* g, int64_t capacity)
{
    if (!ctx || !g) return MRMD_ERR_ARG;
    std::memset(g, 0, sizeof(*g));
    if (capacity < 1) capacity = 1;
    return ensure_layer(ctx, g, capacity, capacity);
}

int mrmd_ghost_layer_free(mrmd_ctx* ctx, mrmd_ghost_layer* g)
{
    if (!g) return MRMD_ERR_ARG;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(g->correspondingRealAtom);
    dfree(g->ghostStart);
    dfree(g->ghostList);
    std::memset(g, 0, sizeof(*g));
    return MRMD_OK;
}

int mrmd_ghost_exchange_real_atoms(mrmd_ctx* ctx, mrmd_atoms* a, const mrmd_subdomain* sd)
{
    if (!ctx || !a || !sd) return MRMD_ERR_ARG;
    if (a->numLocal == 0) return MRMD_OK;
    k_map_into_domain<<<grid_for(ctx, a->numLocal, TB), TB, 0, ctx->stream>>>(
        reinterpret_cast<double4*>(a->pos), a->numLocal, d3(sd->minCorner), d3(sd->maxCorner),
        d3(sd->diameter));
    MRMD_TRY(after_launch(ctx, "map_into_domain"));
    return finish(ctx, "map_into_domain");
}

int mrmd_ghost_create(mrmd_ctx* ctx, mrmd_ghost_layer* g, mrmd_atoms* a, const mrmd_subdomain* sd)
{
    // GhostExchange::createGhostAtomsXYZ, communication/GhostExchange.cpp:171-181
    if (!ctx || !g || !a || !sd) return MRMD_ERR_ARG;
    const int64_t nLocal = a->numLocal;
    MRMD_TRY(ensure_layer(ctx, g, a->capacity > nLocal + 1 ? a->capacity : nLocal + 1, nLocal + 1));
    k_fill_i32<<<grid_for(ctx, g->capacity, TB), TB, 0, ctx->stream>>>(g->correspondingRealAtom,
                                                                        g->capacity, -1);
    MRMD_TRY(after_launch(ctx, "fill_corr"));
    a->numGhost = 0;
    int64_t* total = reinterpret_cast<int64_t*>(ctx->devScalars);
    for (int axis = 0; axis < 3; ++axis)
    {
        const int64_t n = a->numLocal + a->numGhost;
        int64_t* offs = static_cast<int64_t*>(scratch(ctx, sizeof(int64_t) * (size_t)(n + 1)));
        if (!offs) return MRMD_ERR_OOM;
        k_ghost_flags<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(
            reinterpret_cast<const double4*>(a->pos), n, axis, sd->minInnerCorner[axis],
            sd->maxInnerCorner[axis], offs);
        MRMD_TRY(after_launch(ctx, "ghost_flags"));
        MRMD_TRY(scan_exclusive_i64(ctx, offs, offs, n, total));
        int64_t hTotal = 0;
        MRMD_CUDA(ctx, cudaMemcpyAsync(&hTotal, total, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int64_t numLo = hTotal & 0xffffffffLL, numHi = hTotal >> 32;
        const int64_t need = n + numLo + numHi;
        if (need > INT32_MAX) return set_error(ctx, MRMD_ERR_CAPACITY, "more than 2^31 atoms");
        if (need > a->capacity)
        {
            MRMD_TRY(mrmd_atoms_reserve(ctx, a, need + need / 8 + 64));
        }
        MRMD_TRY(ensure_layer(ctx, g, a->capacity, nLocal + 1));
        if (numLo + numHi > 0)
        {
            k_ghost_copy<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(
                *a, g->correspondingRealAtom, n, axis, sd->minInnerCorner[axis], sd->maxInnerCorner[axis],
                sd->diameter[axis], offs, total);
            MRMD_TRY(after_launch(ctx, "ghost_copy"));
        }
        a->numGhost += numLo + numHi;
    }
    g->numLocal = a->numLocal;
    g->numGhost = a->numGhost;
    MRMD_TRY(build_csr(ctx, g, g->numLocal, g->numGhost));
    return finish(ctx, "ghost_create");
}

int mrmd_ghost_update(mrmd_ctx* ctx, const mrmd_ghost_layer* g, mrmd_atoms* a, const mrmd_subdomain* sd)
{
    if (!ctx || !g || !a || !sd) return MRMD_ERR_ARG;
    if (g->numLocal != a->numLocal || g->numGhost != a->numGhost)
        return set_error(ctx, MRMD_ERR_STATE, "ghost layer does not match atoms (recreate ghosts)");
    if (a->numGhost == 0) return MRMD_OK;
    const double delta[3] = {0.1 * sd->diameter[0], 0.1 * sd->diameter[1], 0.1 * sd->diameter[2]};
    k_ghost_update<<<grid_for(ctx, a->numGhost, TB), TB, 0, ctx->stream>>>(
        reinterpret_cast<double4*>(a->pos), g->correspondingRealAtom, a->numLocal, a->numGhost,
        d3(sd->diameter), d3(delta));
    MRMD_TRY(after_launch(ctx, "ghost_update"));
    return finish(ctx, "ghost_update");
}

int mrmd_ghost_reduce_force(mrmd_ctx* ctx, const mrmd_ghost_layer* g, mrmd_atoms* a)
{
    if (!ctx || !g || !a) return MRMD_ERR_ARG;
    if (g->numLocal != a->numLocal || g->numGhost != a->numGhost)
        return set_error(ctx, MRMD_ERR_STATE, "ghost layer does not match atoms (recreate ghosts)");
    if (a->numGhost == 0 || a->numLocal == 0) return MRMD_OK;
    k_ghost_reduce<<<grid_for(ctx, a->numLocal, TB), TB, 0, ctx->stream>>>(
        reinterpret_cast<double4*>(a->force), g->ghostStart, g->ghostList, a->numLocal, a->numGhost);
    MRMD_TRY(after_launch(ctx, "ghost_reduce"));
    return finish(ctx, "ghost_reduce");
}

int mrmd_ghost_layer_download(mrmd_ctx* ctx, const mrmd_ghost_layer* g, int64_t n, int64_t* out)
{
    if (!ctx || !g || !out) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(n >= 0 && n <= g->capacity, ctx, "download size out of range");
    if (n == 0) return MRMD_OK;
    int32_t* tmp = nullptr;
    MRMD_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&tmp), sizeof(int32_t) * (size_t)n));
    cudaError_t e = cudaMemcpyAsync(tmp, g->correspondingRealAtom, sizeof(int32_t) * (size_t)n,
                                    cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess)
        for (int64_t i = 0; i < n; ++i) out[i] = tmp[i];
    cudaFreeHost(tmp);
    return check_cuda(ctx, e, "ghost_layer_download");
}

int mrmd_multires_exchange_real_atoms(mrmd_ctx* ctx, mrmd_molecules* m, mrmd_atoms* a,
                                      const mrmd_subdomain* sd)
{
    if (!ctx || !m || !a || !sd) return MRMD_ERR_ARG;
    if (m->numLocal == 0) return MRMD_OK;
    k_multires_map<<<grid_for(ctx, m->numLocal, TB), TB, 0, ctx->stream>>>(
        *m, reinterpret_cast<double4*>(a->pos), m->numLocal, d3(sd->minCorner), d3(sd->maxCorner),
        d3(sd->diameter));
    MRMD_TRY(after_launch(ctx, "multires_map"));
    return finish(ctx, "multires_map");
}

int mrmd_multires_ghost_create(mrmd_ctx* ctx, mrmd_ghost_layer* g, mrmd_molecules* m, mrmd_atoms* a,
                               const mrmd_subdomain* sd)
{
    // MultiResPeriodicGhostExchange::createGhostAtomsXYZ (:250-265)
    if (!ctx || !g || !m || !a || !sd) return MRMD_ERR_ARG;
    const int64_t nLocal = a->numLocal;
    MRMD_TRY(ensure_layer(ctx, g, a->capacity > nLocal + 1 ? a->capacity : nLocal + 1, nLocal + 1));
    k_fill_i32<<<grid_for(ctx, g->capacity, TB), TB, 0, ctx->stream>>>(g->correspondingRealAtom,
                                                                        g->capacity, -1);
    MRMD_TRY(after_launch(ctx, "fill_corr"));
    m->numGhost = 0;
    a->numGhost = 0;
    int64_t* totals = reinterpret_cast<int64_t*>(ctx->devScalars);
    for (int axis = 0; axis < 3; ++axis)
    {
        const int64_t nM = m->numLocal + m->numGhost;
        const int64_t nA = a->numLocal + a->numGhost;
        int64_t* hi = static_cast<int64_t*>(scratch(ctx, sizeof(int64_t) * 2 * (size_t)(nM + 1)));
        if (!hi) return MRMD_ERR_OOM;
        int64_t* lo = hi + (nM + 1);
        k_multires_flags<<<grid_for(ctx, nM, TB), TB, 0, ctx->stream>>>(
            *m, nM, axis, sd->minInnerCorner[axis], sd->maxInnerCorner[axis], hi, lo);
        MRMD_TRY(after_launch(ctx, "multires_flags"));
        MRMD_TRY(scan_exclusive_i64(ctx, hi, hi, nM, totals));
        MRMD_TRY(scan_exclusive_i64(ctx, lo, lo, nM, totals + 1));
        int64_t h[2] = {0, 0};
        MRMD_CUDA(ctx, cudaMemcpyAsync(h, totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int64_t addM = (h[0] & 0xffffffffLL) + (h[1] & 0xffffffffLL);
        const int64_t addA = (h[0] >> 32) + (h[1] >> 32);
        if (nM + addM > m->capacity) MRMD_TRY(mrmd_molecules_reserve(ctx, m, nM + addM + (nM + addM) / 8 + 64));
        if (nA + addA > a->capacity) MRMD_TRY(mrmd_atoms_reserve(ctx, a, nA + addA + (nA + addA) / 8 + 64));
        MRMD_TRY(ensure_layer(ctx, g, a->capacity, nLocal + 1));
        if (addM > 0)
        {
            k_multires_copy<<<grid_for(ctx, nM, TB), TB, 0, ctx->stream>>>(
                *m, *a, g->correspondingRealAtom, nM, nA, axis, sd->minInnerCorner[axis],
                sd->maxInnerCorner[axis], sd->diameter[axis], hi, lo, totals);
            MRMD_TRY(after_launch(ctx, "multires_copy"));
        }
        m->numGhost += addM;
        a->numGhost += addA;
    }
    g->numLocal = a->numLocal;
    g->numGhost = a->numGhost;
    MRMD_TRY(build_csr(ctx, g, g->numLocal, g->numGhost));
    return finish(ctx, "multires_ghost_create");
}

}  // extern "C"
