// analysis::getKineticEnergy, getSystemMomentum and getPressure on the
// device, as deterministic grid sums (reduce_impl.cuh): one pass over the
// atoms, the result copied back through the context's pinned scalars.
#include "common.cuh"
#include "reduce_impl.cuh"

using namespace mrmd_impl;

namespace
{
constexpr int TB = 256;
constexpr int NOBS = 6;  // local m v.v, local sum v (3), all m v.v, all F.x

__global__ void k_observe(const double4* __restrict__ pos, const double4* __restrict__ vel,
                          const double4* __restrict__ force, const double* __restrict__ mass, int64_t nLocal,
                          int64_t nAll, double* partial, unsigned* ticket, double* out)
{
    double v[NOBS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nAll;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double4 u = vel[i];
        // KineticEnergy.hpp:33-34 / Pressure.cpp:33-34
        const double mvv = mass[i] * (u.x * u.x + u.y * u.y + u.z * u.z);
        if (i < nLocal)
        {
            v[0] += mvv;
            v[1] += u.x;
            v[2] += u.y;
            v[3] += u.z;
        }
        const double4 x = pos[i], f = force[i];
        v[4] += mvv;
        v[5] += f.x * x.x + f.y * x.y + f.z * x.z;  // Pressure.cpp:46 (dot3(F, x))
    }
    grid_sum<NOBS>(v, partial, ticket, out);
}

int observe(mrmd_ctx* ctx, const mrmd_atoms* a, bool ghosts, double* host)
{
    const int64_t nLocal = a->numLocal, nAll = ghosts ? a->numLocal + a->numGhost : a->numLocal;
    const unsigned grid = grid_for(ctx, nAll, TB, 4);
    // partials, then the ticket (zeroed here; reset by the kernel's last block)
    char* s = static_cast<char*>(scratch(ctx, sizeof(double) * NOBS * grid + 256));
    if (!s) return MRMD_ERR_OOM;
    double* partial = reinterpret_cast<double*>(s);
    unsigned* ticket = reinterpret_cast<unsigned*>(s + sizeof(double) * NOBS * grid);
    double* out = ctx->devScalars + 56;
    MRMD_CUDA(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned), ctx->stream));
    k_observe<<<grid, TB, 0, ctx->stream>>>(reinterpret_cast<const double4*>(a->pos),
                                            reinterpret_cast<const double4*>(a->vel),
                                            reinterpret_cast<const double4*>(a->force), a->mass, nLocal, nAll,
                                            partial, ticket, out);
    MRMD_TRY(after_launch(ctx, "observe"));
    MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 56, out, sizeof(double) * NOBS, cudaMemcpyDeviceToHost,
                                   ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < NOBS; ++k) host[k] = ctx->hostScalars[56 + k];
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_kinetic_energy(mrmd_ctx* ctx, const mrmd_atoms* a, double* out)
{
    // analysis/KineticEnergy.hpp:26-39
    if (!ctx || !a || !out) return MRMD_ERR_ARG;
    double h[NOBS];
    MRMD_TRY(observe(ctx, a, false, h));
    *out = 0.5 * h[0];
    return MRMD_OK;
}

int mrmd_system_momentum(mrmd_ctx* ctx, const mrmd_atoms* a, double* out3)
{
    // analysis/SystemMomentum.cpp:21-48
    if (!ctx || !a || !out3) return MRMD_ERR_ARG;
    double h[NOBS];
    MRMD_TRY(observe(ctx, a, false, h));
    for (int d = 0; d < 3; ++d) out3[d] = h[1 + d];
    return MRMD_OK;
}

int mrmd_pressure(mrmd_ctx* ctx, const mrmd_atoms* a, const mrmd_subdomain* sd, double* out)
{
    // analysis/Pressure.cpp:23-51, Subdomain::getVolume (data/Subdomain.cpp:57)
    if (!ctx || !a || !sd || !out) return MRMD_ERR_ARG;
    double h[NOBS];
    MRMD_TRY(observe(ctx, a, true, h));
    const double volume = sd->diameter[0] * sd->diameter[1] * sd->diameter[2];
    *out = (h[4] + h[5]) / (3.0 * volume);
    return MRMD_OK;
}

}  // extern "C"
