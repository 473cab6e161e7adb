// Device storage of data::Atoms / data::Molecules and host transfers.
//
// Vectors are stored as [capacity][4] doubles: one atom's x, y, z (+ pad)
// fill exactly one 32-byte sector, so a neighbour gather or an atomic
// j-force update touches a single sector.
#include <vector>

#include "common.cuh"

using namespace mrmd_impl;

namespace
{
__global__ void k_expand3(const double* __restrict__ src3, double4* __restrict__ dst, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = make_double4(src3[3 * i], src3[3 * i + 1], src3[3 * i + 2], 0.0);
}

__global__ void k_pack3(const double4* __restrict__ src, double* __restrict__ dst3, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double4 v = src[i];
        dst3[3 * i] = v.x;
        dst3[3 * i + 1] = v.y;
        dst3[3 * i + 2] = v.z;
    }
}

__global__ void k_fill4(double4* __restrict__ dst, int64_t n, double v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = make_double4(v, v, v, 0.0);
}

template <typename T>
int realloc_keep(mrmd_ctx* ctx, T*& p, int64_t oldN, int64_t newN, int64_t width)
{
    T* np = nullptr;
    MRMD_TRY(dmalloc(ctx, reinterpret_cast<void**>(&np), sizeof(T) * (size_t)(newN * width)));
    MRMD_CUDA(ctx, cudaMemsetAsync(np, 0, sizeof(T) * (size_t)(newN * width), ctx->stream));
    if (p != nullptr && oldN > 0)
        MRMD_CUDA(ctx, cudaMemcpyAsync(np, p, sizeof(T) * (size_t)(oldN * width),
                                       cudaMemcpyDeviceToDevice, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    dfree(p);
    p = np;
    return MRMD_OK;
}

// host [n][3] -> device [n][4] through a device staging buffer
int upload3(mrmd_ctx* ctx, double* dst4, const double* host3, int64_t n)
{
    if (host3 == nullptr || n == 0) return MRMD_OK;
    double* stage = static_cast<double*>(scratch(ctx, sizeof(double) * 3 * (size_t)n));
    if (!stage) return MRMD_ERR_OOM;
    MRMD_CUDA(ctx, cudaMemcpyAsync(stage, host3, sizeof(double) * 3 * (size_t)n,
                                   cudaMemcpyHostToDevice, ctx->stream));
    k_expand3<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(stage, reinterpret_cast<double4*>(dst4), n);
    MRMD_TRY(after_launch(ctx, "expand3"));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "upload3");
}

int download3(mrmd_ctx* ctx, double* host3, const double* src4, int64_t n)
{
    if (host3 == nullptr || n == 0) return MRMD_OK;
    double* stage = static_cast<double*>(scratch(ctx, sizeof(double) * 3 * (size_t)n));
    if (!stage) return MRMD_ERR_OOM;
    k_pack3<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(reinterpret_cast<const double4*>(src4), stage, n);
    MRMD_TRY(after_launch(ctx, "pack3"));
    MRMD_CUDA(ctx, cudaMemcpyAsync(host3, stage, sizeof(double) * 3 * (size_t)n,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "download3");
}

template <typename T>
int upload1(mrmd_ctx* ctx, T* dst, const T* host, int64_t n)
{
    if (host == nullptr || n == 0) return MRMD_OK;
    MRMD_CUDA(ctx, cudaMemcpyAsync(dst, host, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "upload1");
}

template <typename T>
int download1(mrmd_ctx* ctx, T* host, const T* src, int64_t n)
{
    if (host == nullptr || n == 0) return MRMD_OK;
    MRMD_CUDA(ctx, cudaMemcpyAsync(host, src, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "download1");
}
}  // namespace

extern "C" {

int mrmd_atoms_alloc(mrmd_ctx* ctx, mrmd_atoms* a, int64_t capacity)
{
    if (!ctx || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(capacity >= 0, ctx, "negative capacity");
    std::memset(a, 0, sizeof(*a));
    if (capacity < 1) capacity = 1;
    MRMD_TRY(realloc_keep(ctx, a->pos, 0, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, a->vel, 0, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, a->force, 0, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, a->type, 0, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, a->mass, 0, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, a->charge, 0, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, a->relativeMass, 0, capacity, 1));
    a->capacity = capacity;
    return MRMD_OK;
}

int mrmd_atoms_free(mrmd_ctx* ctx, mrmd_atoms* a)
{
    if (!a) return MRMD_ERR_ARG;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(a->pos);
    dfree(a->vel);
    dfree(a->force);
    dfree(a->type);
    dfree(a->mass);
    dfree(a->charge);
    dfree(a->relativeMass);
    std::memset(a, 0, sizeof(*a));
    return MRMD_OK;
}

int mrmd_atoms_reserve(mrmd_ctx* ctx, mrmd_atoms* a, int64_t capacity)
{
    if (!ctx || !a) return MRMD_ERR_ARG;
    if (capacity <= a->capacity) return MRMD_OK;
    const int64_t old = a->capacity;
    MRMD_TRY(realloc_keep(ctx, a->pos, old, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, a->vel, old, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, a->force, old, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, a->type, old, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, a->mass, old, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, a->charge, old, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, a->relativeMass, old, capacity, 1));
    a->capacity = capacity;
    return MRMD_OK;
}

int mrmd_atoms_upload(mrmd_ctx* ctx, mrmd_atoms* a, int64_t numLocal, int64_t numGhost,
                      const double* pos3, const double* vel3, const double* force3,
                      const int64_t* type, const double* mass, const double* charge,
                      const double* relativeMass)
{
    if (!ctx || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(numLocal >= 0 && numGhost >= 0, ctx, "negative atom count");
    const int64_t n = numLocal + numGhost;
    if (n > a->capacity) MRMD_TRY(mrmd_atoms_reserve(ctx, a, n));
    MRMD_TRY(upload3(ctx, a->pos, pos3, n));
    MRMD_TRY(upload3(ctx, a->vel, vel3, n));
    MRMD_TRY(upload3(ctx, a->force, force3, n));
    if (type != nullptr && n > 0)
    {
        std::vector<int32_t> t32((size_t)n);
        for (int64_t i = 0; i < n; ++i)
        {
            if (type[i] < 0 || type[i] > INT32_MAX)
                return set_error(ctx, MRMD_ERR_ARG, "atom type %lld out of range", (long long)type[i]);
            t32[(size_t)i] = (int32_t)type[i];
        }
        MRMD_TRY(upload1(ctx, a->type, t32.data(), n));
    }
    MRMD_TRY(upload1(ctx, a->mass, mass, n));
    MRMD_TRY(upload1(ctx, a->charge, charge, n));
    MRMD_TRY(upload1(ctx, a->relativeMass, relativeMass, n));
    a->numLocal = numLocal;
    a->numGhost = numGhost;
    return MRMD_OK;
}

int mrmd_atoms_download(mrmd_ctx* ctx, const mrmd_atoms* a, int64_t n, double* pos3, double* vel3,
                        double* force3, int64_t* type, double* mass, double* charge,
                        double* relativeMass)
{
    if (!ctx || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(n >= 0 && n <= a->capacity, ctx, "download size out of range");
    MRMD_TRY(download3(ctx, pos3, a->pos, n));
    MRMD_TRY(download3(ctx, vel3, a->vel, n));
    MRMD_TRY(download3(ctx, force3, a->force, n));
    if (type != nullptr && n > 0)
    {
        std::vector<int32_t> t32((size_t)n);
        MRMD_TRY(download1(ctx, t32.data(), a->type, n));
        for (int64_t i = 0; i < n; ++i) type[i] = t32[(size_t)i];
    }
    MRMD_TRY(download1(ctx, mass, a->mass, n));
    MRMD_TRY(download1(ctx, charge, a->charge, n));
    MRMD_TRY(download1(ctx, relativeMass, a->relativeMass, n));
    return MRMD_OK;
}

int mrmd_atoms_set_force(mrmd_ctx* ctx, mrmd_atoms* a, int64_t n, double val)
{
    if (!ctx || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(n >= 0 && n <= a->capacity, ctx, "set_force size out of range");
    if (n == 0) return MRMD_OK;
    k_fill4<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(reinterpret_cast<double4*>(a->force), n, val);
    MRMD_TRY(after_launch(ctx, "set_force"));
    return finish(ctx, "set_force");
}

// -------------------------------------------------------------- molecules --

int mrmd_molecules_alloc(mrmd_ctx* ctx, mrmd_molecules* m, int64_t capacity)
{
    if (!ctx || !m) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(capacity >= 0, ctx, "negative capacity");
    std::memset(m, 0, sizeof(*m));
    if (capacity < 1) capacity = 1;
    MRMD_TRY(realloc_keep(ctx, m->pos, 0, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, m->force, 0, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, m->lambda, 0, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, m->modulatedLambda, 0, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, m->gradLambda, 0, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, m->atomsOffset, 0, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, m->numAtoms, 0, capacity, 1));
    m->capacity = capacity;
    return MRMD_OK;
}

int mrmd_molecules_free(mrmd_ctx* ctx, mrmd_molecules* m)
{
    if (!m) return MRMD_ERR_ARG;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(m->pos);
    dfree(m->force);
    dfree(m->lambda);
    dfree(m->modulatedLambda);
    dfree(m->gradLambda);
    dfree(m->atomsOffset);
    dfree(m->numAtoms);
    std::memset(m, 0, sizeof(*m));
    return MRMD_OK;
}

int mrmd_molecules_reserve(mrmd_ctx* ctx, mrmd_molecules* m, int64_t capacity)
{
    if (!ctx || !m) return MRMD_ERR_ARG;
    if (capacity <= m->capacity) return MRMD_OK;
    const int64_t old = m->capacity;
    MRMD_TRY(realloc_keep(ctx, m->pos, old, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, m->force, old, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, m->lambda, old, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, m->modulatedLambda, old, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, m->gradLambda, old, capacity, 4));
    MRMD_TRY(realloc_keep(ctx, m->atomsOffset, old, capacity, 1));
    MRMD_TRY(realloc_keep(ctx, m->numAtoms, old, capacity, 1));
    m->capacity = capacity;
    return MRMD_OK;
}

int mrmd_molecules_upload(mrmd_ctx* ctx, mrmd_molecules* m, int64_t numLocal, int64_t numGhost,
                          const double* pos3, const double* force3, const double* lambda,
                          const double* modulatedLambda, const double* gradLambda3,
                          const int64_t* atomsOffset, const int64_t* numAtoms)
{
    if (!ctx || !m) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(numLocal >= 0 && numGhost >= 0, ctx, "negative molecule count");
    const int64_t n = numLocal + numGhost;
    if (n > m->capacity) MRMD_TRY(mrmd_molecules_reserve(ctx, m, n));
    MRMD_TRY(upload3(ctx, m->pos, pos3, n));
    MRMD_TRY(upload3(ctx, m->force, force3, n));
    MRMD_TRY(upload1(ctx, m->lambda, lambda, n));
    MRMD_TRY(upload1(ctx, m->modulatedLambda, modulatedLambda, n));
    MRMD_TRY(upload3(ctx, m->gradLambda, gradLambda3, n));
    MRMD_TRY(upload1(ctx, m->atomsOffset, atomsOffset, n));
    MRMD_TRY(upload1(ctx, m->numAtoms, numAtoms, n));
    m->numLocal = numLocal;
    m->numGhost = numGhost;
    return MRMD_OK;
}

int mrmd_molecules_download(mrmd_ctx* ctx, const mrmd_molecules* m, int64_t n, double* pos3,
                            double* force3, double* lambda, double* modulatedLambda,
                            double* gradLambda3, int64_t* atomsOffset, int64_t* numAtoms)
{
    if (!ctx || !m) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(n >= 0 && n <= m->capacity, ctx, "download size out of range");
    MRMD_TRY(download3(ctx, pos3, m->pos, n));
    MRMD_TRY(download3(ctx, force3, m->force, n));
    MRMD_TRY(download1(ctx, lambda, m->lambda, n));
    MRMD_TRY(download1(ctx, modulatedLambda, m->modulatedLambda, n));
    MRMD_TRY(download3(ctx, gradLambda3, m->gradLambda, n));
    MRMD_TRY(download1(ctx, atomsOffset, m->atomsOffset, n));
    MRMD_TRY(download1(ctx, numAtoms, m->numAtoms, n));
    return MRMD_OK;
}

int mrmd_molecules_set_force(mrmd_ctx* ctx, mrmd_molecules* m, int64_t n, double val)
{
    if (!ctx || !m) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(n >= 0 && n <= m->capacity, ctx, "set_force size out of range");
    if (n == 0) return MRMD_OK;
    k_fill4<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(reinterpret_cast<double4*>(m->force), n, val);
    MRMD_TRY(after_launch(ctx, "molecules_set_force"));
    return finish(ctx, "molecules_set_force");
}

}  // extern "C"
