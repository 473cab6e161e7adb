// Context, error reporting, scratch memory and exclusive scans.
#include <cstdarg>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace mrmd_impl
{
int set_error(mrmd_ctx* ctx, int code, const char* fmt, ...)
{
    if (ctx != nullptr)
    {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->lastError, sizeof(ctx->lastError), fmt, ap);
        va_end(ap);
    }
    return code;
}

int check_cuda(mrmd_ctx* ctx, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return MRMD_OK;
    if (e == cudaErrorMemoryAllocation)
    {
        cudaGetLastError();
        return set_error(ctx, MRMD_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    }
    return set_error(ctx, MRMD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int after_launch(mrmd_ctx* ctx, const char* what)
{
    ctx->launches++;
    return check_cuda(ctx, cudaGetLastError(), what);
}

int finish(mrmd_ctx* ctx, const char* what)
{
    if (!ctx->sync) return MRMD_OK;
    MRMD_TRY(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), what));
    return bounds_check(ctx);
}

namespace
{
struct BoundsTU
{
    const char* file;
    int (*read)(long long*);
    int (*clear)();
};

std::vector<BoundsTU>& bounds_registry()
{
    static std::vector<BoundsTU> r;
    return r;
}
}  // namespace

void bounds_register(const char* file, int (*read)(long long*), int (*clear)())
{
    bounds_registry().push_back(BoundsTU{file, read, clear});
}

int bounds_check(mrmd_ctx* ctx)
{
#ifdef MRMD_BOUNDS_CHECK
    for (const BoundsTU& t : bounds_registry())
    {
        long long rec[3] = {0, 0, 0};
        if (t.read(rec) != 0) return set_error(ctx, MRMD_ERR_CUDA, "bounds record of %s unreadable", t.file);
        if (rec[0] == 0) continue;
        t.clear();
        const char* base = std::strrchr(t.file, '/');
        return set_error(ctx, MRMD_ERR_BOUNDS, "bounds check: %s:%lld index %lld outside [0, %lld)",
                         base ? base + 1 : t.file, rec[0] - 1, rec[1], rec[2]);
    }
#else
    (void)ctx;
#endif
    return MRMD_OK;
}

int dmalloc(mrmd_ctx* ctx, void** p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        *p = nullptr;
        return set_error(ctx, MRMD_ERR_OOM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return MRMD_OK;
}

void dfree(void* p)
{
    if (p) cudaFree(p);
}

int h2d(mrmd_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    if (bytes == 0) return MRMD_OK;
    MRMD_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "h2d");
}

int d2h(mrmd_ctx* ctx, void* dst, const void* src, size_t bytes)
{
    if (bytes == 0) return MRMD_OK;
    MRMD_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "d2h");
}

int dzero(mrmd_ctx* ctx, void* p, size_t bytes)
{
    if (bytes == 0) return MRMD_OK;
    MRMD_CUDA(ctx, cudaMemsetAsync(p, 0, bytes, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "dzero");
}

static void* grow_buffer(mrmd_ctx* ctx, void*& buf, size_t& have, size_t bytes)
{
    if (bytes <= have) return buf;
    size_t nb = bytes + bytes / 4 + (1 << 20);
    cudaStreamSynchronize(ctx->stream);
    dfree(buf);
    buf = nullptr;
    have = 0;
    if (dmalloc(ctx, &buf, nb) != MRMD_OK) return nullptr;
    have = nb;
    return buf;
}

void* scratch(mrmd_ctx* ctx, size_t bytes)
{
    return grow_buffer(ctx, ctx->scratch, ctx->scratchBytes, bytes);
}

// ------------------------------------------------------------------ scan --
// Three-phase exclusive scan: per-tile scan with tile totals, scan of the
// tile totals (recursively), add offsets.  Tiles are 1024 items handled by
// 256 threads x 4 items.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

template <typename T>
__global__ void k_scan_tiles(const T* __restrict__ in, T* __restrict__ out, int64_t n,
                             T* __restrict__ tileSums)
{
    __shared__ T warpSums[SCAN_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    T v[SCAN_ITEMS];
    T local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        v[k] = (base + k < n) ? in[base + k] : T(0);
        local += v[k];
    }
    T incl = warp_incl_scan(local);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 31) warpSums[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        T w = lane < SCAN_THREADS / 32 ? warpSums[lane] : T(0);
        w = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) warpSums[lane] = w;
    }
    __syncthreads();
    T prefix = (warp > 0 ? warpSums[warp - 1] : T(0)) + incl - local;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        if (base + k < n) out[base + k] = prefix;
        prefix += v[k];
    }
    if (threadIdx.x == SCAN_THREADS - 1) tileSums[blockIdx.x] = prefix;
}

template <typename T>
__global__ void k_scan_add(T* __restrict__ out, int64_t n, const T* __restrict__ tileOffsets)
{
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    const T off = tileOffsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) out[base + k] += off;
}

template <typename T>
__global__ void k_scan_total(const T* __restrict__ tileSums, const T* __restrict__ tileOffsets,
                             int64_t tiles, T* __restrict__ total)
{
    *total = tileOffsets[tiles - 1] + tileSums[tiles - 1];
}

template <typename T>
static int scan_rec(mrmd_ctx* ctx, const T* in, T* out, int64_t n, T* total, char* sbuf)
{
    if (n <= 0)
    {
        if (total) MRMD_CUDA(ctx, cudaMemsetAsync(total, 0, sizeof(T), ctx->stream));
        return MRMD_OK;
    }
    const int64_t tiles = div_up(n, SCAN_TILE);
    T* tileSums = reinterpret_cast<T*>(sbuf);
    T* tileOffsets = tileSums + tiles;
    char* next = reinterpret_cast<char*>(tileOffsets + tiles);
    next = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(next) + 255) & ~uintptr_t(255));
    k_scan_tiles<T><<<(unsigned)tiles, SCAN_THREADS, 0, ctx->stream>>>(in, out, n, tileSums);
    MRMD_TRY(after_launch(ctx, "scan_tiles"));
    if (tiles > 1)
    {
        MRMD_TRY(scan_rec<T>(ctx, tileSums, tileOffsets, tiles, nullptr, next));
        k_scan_add<T><<<(unsigned)tiles, SCAN_THREADS, 0, ctx->stream>>>(out, n, tileOffsets);
        MRMD_TRY(after_launch(ctx, "scan_add"));
    }
    else
    {
        MRMD_CUDA(ctx, cudaMemsetAsync(tileOffsets, 0, sizeof(T), ctx->stream));
    }
    if (total)
    {
        k_scan_total<T><<<1, 1, 0, ctx->stream>>>(tileSums, tileOffsets, tiles, total);
        MRMD_TRY(after_launch(ctx, "scan_total"));
    }
    return MRMD_OK;
}

template <typename T>
static size_t scan_scratch_bytes(int64_t n)
{
    size_t b = 0;
    while (n > 0)
    {
        int64_t tiles = div_up(n, SCAN_TILE);
        b += 2 * tiles * sizeof(T) + 512;
        if (tiles <= 1) break;
        n = tiles;
    }
    return b + 1024;
}

int scan_exclusive_i64(mrmd_ctx* ctx, const int64_t* in, int64_t* out, int64_t n, int64_t* total)
{
    char* s = static_cast<char*>(
        grow_buffer(ctx, ctx->scanScratch, ctx->scanScratchBytes, scan_scratch_bytes<int64_t>(n)));
    if (!s) return MRMD_ERR_OOM;
    return scan_rec<int64_t>(ctx, in, out, n, total, s);
}

int scan_exclusive_i32(mrmd_ctx* ctx, const int32_t* in, int32_t* out, int64_t n, int32_t* total)
{
    char* s = static_cast<char*>(
        grow_buffer(ctx, ctx->scanScratch, ctx->scanScratchBytes, scan_scratch_bytes<int32_t>(n)));
    if (!s) return MRMD_ERR_OOM;
    return scan_rec<int32_t>(ctx, in, out, n, total, s);
}
}  // namespace mrmd_impl

using namespace mrmd_impl;

extern "C" {

const char* mrmd_version(void) { return "mrmd_gb300 0.1.0 (sm_103a)"; }

int mrmd_ctx_create(mrmd_ctx** out, int device)
{
    if (out == nullptr) return MRMD_ERR_ARG;
    *out = nullptr;
    mrmd_ctx* ctx = new mrmd_ctx();
    ctx->device = device;
    int rc = check_cuda(ctx, cudaSetDevice(device), "cudaSetDevice");
    if (rc == MRMD_OK) rc = check_cuda(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream");
    if (rc == MRMD_OK)
        rc = check_cuda(ctx, cudaDeviceGetAttribute(&ctx->numSMs, cudaDevAttrMultiProcessorCount, device),
                        "attr");
    if (rc == MRMD_OK)
        rc = check_cuda(ctx, cudaMallocHost(reinterpret_cast<void**>(&ctx->hostScalars), 64 * sizeof(double)),
                        "pinned");
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&ctx->devScalars), 64 * sizeof(double));
    if (rc != MRMD_OK)
    {
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->hostScalars) cudaFreeHost(ctx->hostScalars);
        delete ctx;
        return rc;
    }
    *out = ctx;
    return MRMD_OK;
}

int mrmd_ctx_destroy(mrmd_ctx* ctx)
{
    if (!ctx) return MRMD_OK;
    cudaStreamSynchronize(ctx->stream);
    dfree(ctx->scratch);
    dfree(ctx->scanScratch);
    dfree(ctx->devScalars);
    if (ctx->hostScalars) cudaFreeHost(ctx->hostScalars);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MRMD_OK;
}

int mrmd_ctx_sync(mrmd_ctx* ctx)
{
    if (!ctx) return MRMD_ERR_ARG;
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "sync");
}

int mrmd_ctx_set_sync(mrmd_ctx* ctx, int sync)
{
    if (!ctx) return MRMD_ERR_ARG;
    ctx->sync = sync ? 1 : 0;
    return MRMD_OK;
}

void* mrmd_ctx_stream(mrmd_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

const char* mrmd_ctx_last_error(mrmd_ctx* ctx) { return ctx ? ctx->lastError : "null context"; }

int mrmd_bounds_checked(void)
{
#ifdef MRMD_BOUNDS_CHECK
    return 1;
#else
    return 0;
#endif
}

int64_t mrmd_ctx_launch_count(mrmd_ctx* ctx) { return ctx ? ctx->launches : 0; }

int mrmd_subdomain_init(mrmd_subdomain* sd, const double* minCorner, const double* maxCorner,
                        const double* ghost)
{
    // data/Subdomain.hpp:41-62
    if (!sd || !minCorner || !maxCorner || !ghost) return MRMD_ERR_ARG;
    for (int d = 0; d < 3; ++d)
    {
        if (!(ghost[d] >= 0.0)) return MRMD_ERR_ARG;
        sd->minCorner[d] = minCorner[d];
        sd->maxCorner[d] = maxCorner[d];
        sd->ghostLayerThickness[d] = ghost[d];
        sd->minGhostCorner[d] = minCorner[d] - ghost[d];
        sd->maxGhostCorner[d] = maxCorner[d] + ghost[d];
        sd->minInnerCorner[d] = minCorner[d] + ghost[d];
        sd->maxInnerCorner[d] = maxCorner[d] - ghost[d];
        sd->diameter[d] = maxCorner[d] - minCorner[d];
        sd->diameterWithGhostLayer[d] = maxCorner[d] - minCorner[d] + 2.0 * ghost[d];
    }
    return MRMD_OK;
}

}  // extern "C"
