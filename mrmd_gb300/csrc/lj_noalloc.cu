// The mixed-form LJ pair force without any allocation.
//
// mrmd_lj_apply(..., MRMD_PREC_MIXED, ...) keeps the FP32 split
// coordinates of every atom in context scratch memory that it grows with
// cudaMalloc on demand.  Some callers cannot allocate device memory while
// they run: a host loop that has already handed all free device memory to
// another allocator (a framework's caching allocator or a pre-sized memory
// pool), or a time-critical step loop that may not take the
// synchronisation a cudaMalloc / cudaFree implies.  This entry point uses
// a fixed scratch array in the library's own device memory instead, sized
// at build time for MRMD_LJ_NOALLOC_MAX_ATOMS atoms (local + ghost).
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds it (8 MiB + 256 B) until the process exits.  Host code only
// sees a host-side stand-in under that name, so the device address is
// fetched once per device with cudaGetSymbolAddress, with that device
// current, the first time this entry point runs on it; that first call
// should therefore come before any stream capture.  All calls share the
// array and it keeps the last call's contents: the energy/virial
// accumulators are cleared at the start of every call, and calls that
// overlap on the GPU (other streams, other host threads) race on it.
#include <mutex>

#include "common.cuh"
#include "lj_impl.cuh"
#include "lj_mixed.cuh"
#include "nlist_impl.cuh"

using namespace mrmd_impl;

namespace
{
// [0, 256): energy and virial accumulators (2 doubles); then hi[max], lo[max]
constexpr size_t NOALLOC_HEADER = 256;
constexpr size_t NOALLOC_BYTES = NOALLOC_HEADER + 2 * sizeof(float4) * (size_t)MRMD_LJ_NOALLOC_MAX_ATOMS;

static __device__ __align__(256) unsigned char g_lj_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void* g_addr[MAX_DEVICES] = {nullptr};

// Device address of the scratch array on ctx->device (looked up once).
int noalloc_scratch(mrmd_ctx* ctx, unsigned char** out)
{
    if (ctx->device < 0 || ctx->device >= MAX_DEVICES) return set_error(ctx, MRMD_ERR_ARG, "device id out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_addr[ctx->device] == nullptr)
    {
        int cur = -1;
        MRMD_CUDA(ctx, cudaGetDevice(&cur));
        if (cur != ctx->device) MRMD_CUDA(ctx, cudaSetDevice(ctx->device));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_lj_noalloc_scratch);
        if (cur != ctx->device) cudaSetDevice(cur);
        MRMD_TRY(check_cuda(ctx, e, "cudaGetSymbolAddress(g_lj_noalloc_scratch)"));
        g_addr[ctx->device] = p;
    }
    *out = static_cast<unsigned char*>(g_addr[ctx->device]);
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_lj_apply_mixed_noalloc(mrmd_ctx* ctx, mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl,
                                const mrmd_pred* pred, double* energy, double* virial)
{
    if (!ctx || !lj || !a || !nl) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(pred_valid(pred), ctx, "bad predicate");
    MRMD_TRY(check_list_fits(ctx, nl, a->numLocal, a->numLocal + a->numGhost));
    if (lj->numTypes > 1) return set_error(ctx, MRMD_ERR_ARG, "mixed precision supports one atom type");
    const int64_t nAll = a->numLocal + a->numGhost;
    if (nAll > MRMD_LJ_NOALLOC_MAX_ATOMS)
        return set_error(ctx, MRMD_ERR_CAPACITY,
                         "mrmd_lj_apply_mixed_noalloc: %lld atoms (local + ghost) exceed the fixed scratch of %lld "
                         "atoms; use mrmd_lj_apply",
                         (long long)nAll, (long long)MRMD_LJ_NOALLOC_MAX_ATOMS);
    unsigned char* base = nullptr;
    MRMD_TRY(noalloc_scratch(ctx, &base));
    double* ev = reinterpret_cast<double*>(base);
    float4* hi = reinterpret_cast<float4*>(base + NOALLOC_HEADER);
    float4* lo = hi + MRMD_LJ_NOALLOC_MAX_ATOMS;
    MRMD_CUDA(ctx, cudaMemsetAsync(ev, 0, 2 * sizeof(double), ctx->stream));
    if (nl->rows > 0)
    {
        MRMD_TRY(split_coords(ctx, a->pos, nAll, split_params_for(nl), hi, lo));
        MRMD_TRY(lj_mixed_half(ctx, hi, lo, lj, a, nl, pred, ev));
    }
    if (energy || virial)
    {
        MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 48, ev, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (energy) *energy = ctx->hostScalars[48];
        if (virial) *virial = ctx->hostScalars[49];
        return MRMD_OK;
    }
    return finish(ctx, "lj_apply_mixed_noalloc");
}

}  // extern "C"
