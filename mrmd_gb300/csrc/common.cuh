// Internal helpers shared by the CUDA translation units of libmrmd_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "mrmd_gb300.h"

struct mrmd_ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    int sync = 1;
    int numSMs = 0;
    int64_t launches = 0;
    char lastError[512] = {0};
    // growable device scratch (reductions, scans); never freed while a
    // captured graph may reference it
    void* scratch = nullptr;
    size_t scratchBytes = 0;
    // separate scratch used only inside the scan helpers, so that a caller's
    // scratch pointer stays valid across a scan
    void* scanScratch = nullptr;
    size_t scanScratchBytes = 0;
    // pinned host staging for scalars read back after a kernel
    double* hostScalars = nullptr;  // 64 doubles
    double* devScalars = nullptr;   // 64 doubles on the device
};

namespace mrmd_impl
{
int set_error(mrmd_ctx* ctx, int code, const char* fmt, ...);

// Returns MRMD_ERR_CUDA with a message when `e` is an error.
int check_cuda(mrmd_ctx* ctx, cudaError_t e, const char* what);

// Launch accounting + last-error check after a kernel launch.
int after_launch(mrmd_ctx* ctx, const char* what);

// Synchronise when the context is in synchronous mode.
int finish(mrmd_ctx* ctx, const char* what);

// Scratch memory of at least `bytes` (contents undefined).
void* scratch(mrmd_ctx* ctx, size_t bytes);

int dmalloc(mrmd_ctx* ctx, void** p, size_t bytes);
void dfree(void* p);

// Synchronous copies and fills ordered with the context stream (which is
// non-blocking, so plain cudaMemcpy/cudaMemset on the legacy stream would
// not be ordered with its kernels).
int h2d(mrmd_ctx* ctx, void* dst, const void* src, size_t bytes);
int d2h(mrmd_ctx* ctx, void* dst, const void* src, size_t bytes);
int dzero(mrmd_ctx* ctx, void* p, size_t bytes);

inline int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Grid size for a grid-stride kernel over n items: a multiple of the SM
// count, capped so that every CTA has work.
inline unsigned grid_for(const mrmd_ctx* ctx, int64_t n, int block, int ctasPerSM = 8)
{
    int64_t need = div_up(n > 0 ? n : 1, block);
    int64_t cap = (int64_t)ctx->numSMs * ctasPerSM;
    return (unsigned)(need < cap ? need : cap);
}

// Exclusive scan of int64 values (in and out may alias).  total (device,
// may be null) receives the sum.  Uses ctx scratch.
int scan_exclusive_i64(mrmd_ctx* ctx, const int64_t* in, int64_t* out, int64_t n, int64_t* total);
int scan_exclusive_i32(mrmd_ctx* ctx, const int32_t* in, int32_t* out, int64_t n, int32_t* total);
}  // namespace mrmd_impl

#define MRMD_CHECK_ARG(cond, ctx, msg)                                             \
    do                                                                              \
    {                                                                               \
        if (!(cond)) return mrmd_impl::set_error((ctx), MRMD_ERR_ARG, "%s", (msg)); \
    } while (0)

#define MRMD_TRY(expr)              \
    do                              \
    {                               \
        int _rc = (expr);           \
        if (_rc != MRMD_OK) return _rc; \
    } while (0)

#define MRMD_CUDA(ctx, expr) MRMD_TRY(mrmd_impl::check_cuda((ctx), (expr), #expr))

// ------------------------------------------------------------ device side --

namespace mrmd_dev
{
// Neighbour lists are stored in tiles of 32 rows: entry k of row i lives at
// (i / 32) * 32 * cap + 32 * k + i % 32, so slot k of a warp's 32 rows is one
// 128-byte line and a warp's whole list is one compact 32 x cap tile.
__device__ __forceinline__ int64_t nbr_row(int64_t i, int64_t cap) { return (i >> 5) * (cap << 5) + (i & 31); }

// read-only 32-byte load of one atom sector as two 128-bit loads
__device__ __forceinline__ double4 ldg4(const double4* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return make_double4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of two doubles, result valid in thread 0.  smem >= 2*32 doubles.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* smem)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0)
    {
        smem[warp] = a;
        smem[32 + warp] = b;
    }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (warp == 0)
    {
        a = lane < nw ? smem[lane] : 0.0;
        b = lane < nw ? smem[32 + lane] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
    }
}

// atomicMax for non-negative doubles via their bit pattern (IEEE ordering
// of non-negative values equals integer ordering).
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v)
{
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

struct Pred
{
    int32_t kind;
    int32_t axis;
    double center, slabMin, slabMax, tolerance;
};

__device__ __forceinline__ bool in_symmetric_slab(const Pred& p, double c)
{
    // util/IsInSymmetricSlab.hpp:33-41
    const double absDx = fabs(c - p.center);
    return (absDx >= p.slabMin - p.tolerance && absDx <= p.slabMax + p.tolerance);
}

__device__ __forceinline__ bool pred1(const Pred& p, double x, double y, double z)
{
    if (p.kind == MRMD_PRED_ALWAYS) return true;
    const double c = p.axis == 0 ? x : (p.axis == 1 ? y : z);
    if (p.kind == MRMD_PRED_IN_SLAB) return in_symmetric_slab(p, c);
    if (p.kind == MRMD_PRED_IN_OPEN_INTERVAL) return c > p.slabMin && c < p.slabMax;
    return true;
}

__device__ __forceinline__ bool pred_coord(const Pred& p, double c)
{
    if (p.kind == MRMD_PRED_ALWAYS) return true;
    if (p.kind == MRMD_PRED_IN_SLAB) return in_symmetric_slab(p, c);
    if (p.kind == MRMD_PRED_IN_OPEN_INTERVAL) return c > p.slabMin && c < p.slabMax;
    return true;
}

__device__ __forceinline__ bool pred2(const Pred& p, double x1, double y1, double z1, double x2,
                                      double y2, double z2)
{
    if (p.kind == MRMD_PRED_ALWAYS) return true;
    const double c1 = p.axis == 0 ? x1 : (p.axis == 1 ? y1 : z1);
    const double c2 = p.axis == 0 ? x2 : (p.axis == 1 ? y2 : z2);
    const bool a = in_symmetric_slab(p, c1);
    const bool b = in_symmetric_slab(p, c2);
    if (p.kind == MRMD_PRED_EITHER_IN_SLAB) return a || b;
    if (p.kind == MRMD_PRED_BOTH_IN_SLAB) return a && b;
    return true;
}
}  // namespace mrmd_dev

// ------------------------------------------------- bounds-checked build --
// Compiled with -DMRMD_BOUNDS_CHECK (mrmd_gb300/build.py --bounds-check), every
// MRMD_IN_BOUNDS(idx, n) tests 0 <= idx < n before the access it guards; the
// first violation of a translation unit is recorded (source line, index,
// bound) and the guarded access is skipped, so the kernel completes and the
// host reports MRMD_ERR_BOUNDS at its next synchronisation.  In the normal
// build the macro is `true` and costs nothing.
#ifdef MRMD_BOUNDS_CHECK
namespace mrmd_dev
{
// [0] source line + 1 (0: no violation), [1] index, [2] bound; one copy per
// translation unit (internal linkage)
static __device__ long long g_bounds_rec[3];

__device__ __noinline__ inline bool bounds_fail(long long idx, long long n, int line)
{
    if (atomicCAS(reinterpret_cast<unsigned long long*>(&g_bounds_rec[0]), 0ull,
                  (unsigned long long)(line + 1)) == 0ull)
    {
        g_bounds_rec[1] = idx;
        g_bounds_rec[2] = n;
    }
    return false;
}
}  // namespace mrmd_dev
#define MRMD_IN_BOUNDS(idx, n)                                                     \
    ((((long long)(idx)) >= 0 && ((long long)(idx)) < ((long long)(n))) ||        \
     mrmd_dev::bounds_fail((long long)(idx), (long long)(n), __LINE__))

namespace mrmd_impl
{
void bounds_register(const char* file, int (*read)(long long*), int (*clear)());
}
namespace
{
int bounds_read_tu(long long* out)
{
    return cudaMemcpyFromSymbol(out, mrmd_dev::g_bounds_rec, 3 * sizeof(long long)) == cudaSuccess ? 0 : -1;
}
int bounds_clear_tu()
{
    const long long z[3] = {0, 0, 0};
    return cudaMemcpyToSymbol(mrmd_dev::g_bounds_rec, z, sizeof(z)) == cudaSuccess ? 0 : -1;
}
struct BoundsRegistrar
{
    BoundsRegistrar() { mrmd_impl::bounds_register(__BASE_FILE__, &bounds_read_tu, &bounds_clear_tu); }
};
BoundsRegistrar g_boundsRegistrar;
}  // namespace
#else
#define MRMD_IN_BOUNDS(idx, n) true
#endif

namespace mrmd_impl
{
// MRMD_ERR_BOUNDS with the first recorded violation of any translation unit
// (bounds-checked build; MRMD_OK otherwise).  Call after a synchronisation.
int bounds_check(mrmd_ctx* ctx);
}

inline mrmd_dev::Pred to_dev_pred(const mrmd_pred* p)
{
    mrmd_dev::Pred d{};
    if (p == nullptr)
    {
        d.kind = MRMD_PRED_ALWAYS;
        return d;
    }
    d.kind = p->kind;
    d.axis = p->axis;
    d.center = p->center;
    d.slabMin = p->slabMin;
    d.slabMax = p->slabMax;
    d.tolerance = p->tolerance;
    return d;
}

inline bool pred_valid(const mrmd_pred* p)
{
    return p == nullptr || (p->kind >= 0 && p->kind <= 4 && p->axis >= 0 && p->axis <= 2);
}
