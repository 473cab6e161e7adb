// action::VelocityVerlet and action::VelocityVerletLangevinThermostat.
//
// Every FP64 operation is written with an explicit round-to-nearest
// intrinsic in the reference's order, so no multiply-add is fused and the
// result is bit-identical to the reference's arithmetic.
#include "common.cuh"
#include "integrate_impl.cuh"

using namespace mrmd_impl;

namespace mrmd_impl
{
__global__ void k_vv_pre(double4* __restrict__ pos, double4* __restrict__ vel, const double4* __restrict__ force,
                         const double* __restrict__ mass, int64_t n, double dtHalf, double dt,
                         double* __restrict__ maxDistSqr)
{
    double m2 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        m2 = fmax(m2, vv_pre_one(pos[i], vel[i], force[i], mass[i], dtHalf, dt, pos + i, vel + i));
    m2 = mrmd_dev::warp_max(m2);
    if ((threadIdx.x & 31) == 0) mrmd_dev::atomic_max_nonneg(maxDistSqr, m2);
}

__global__ void k_vv_post(double4* __restrict__ vel, const double4* __restrict__ force,
                          const double* __restrict__ mass, int64_t n, double dtHalf)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        double4 v = vel[i];
        kick(v, force[i], __ddiv_rn(dtHalf, mass[i]));
        vel[i] = v;
    }
}

__global__ void k_langevin_pre(double4* __restrict__ pos, double4* __restrict__ vel,
                               const double4* __restrict__ force, const double* __restrict__ mass, int64_t n,
                               double dtHalf, double dt, double zeta, double temperature, uint64_t seed,
                               uint64_t step, mrmd_dev::Pred pred, double* __restrict__ maxDistSqr)
{
    // action/VelocityVerletLangevinThermostat.hpp:64-113
    double m2 = 0.0;
    OUCoef ou;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        double4 x = pos[i], v = vel[i];
        const double4 f = force[i];
        const double m = mass[i];
        const double4 x0 = x;
        kick(v, f, __ddiv_rn(dtHalf, m));
        drift(x, v, dtHalf);
        if (mrmd_dev::pred1(pred, x.x, x.y, x.z))
        {
            double g[3];
            normal3(seed, step, (uint64_t)i, g);
            ou.update(m, dt, zeta, temperature);
            ornstein_uhlenbeck(v, ou, g);
        }
        drift(x, v, dtHalf);
        pos[i] = x;
        vel[i] = v;
        m2 = fmax(m2, disp_sqr(x0, x));
    }
    m2 = mrmd_dev::warp_max(m2);
    if ((threadIdx.x & 31) == 0) mrmd_dev::atomic_max_nonneg(maxDistSqr, m2);
}
}  // namespace mrmd_impl

namespace mrmd_impl
{
// Langevin pre-force step without reading the displacement back; dMax
// (device) receives the max |dx|^2 via atomicMax (caller zeroes it).
int langevin_pre_async(mrmd_ctx* ctx, mrmd_atoms* a, double dt, double zeta, double temperature, uint64_t seed,
                       uint64_t step, const mrmd_pred* pred, double* dMax)
{
    const int64_t n = a->numLocal;
    if (n == 0) return MRMD_OK;
    k_langevin_pre<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
        reinterpret_cast<double4*>(a->pos), reinterpret_cast<double4*>(a->vel),
        reinterpret_cast<const double4*>(a->force), a->mass, n, 0.5 * dt, dt, zeta, temperature, seed, step,
        to_dev_pred(pred), dMax);
    return after_launch(ctx, "langevin_pre");
}
}  // namespace mrmd_impl

static int read_max_disp(mrmd_ctx* ctx, double* dMax, double* out)
{
    if (!out) return finish(ctx, "integrate");
    MRMD_CUDA(ctx, cudaMemcpyAsync(ctx->hostScalars + 24, dMax, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out = std::sqrt(ctx->hostScalars[24]);
    return MRMD_OK;
}

extern "C" {

int mrmd_vv_pre(mrmd_ctx* ctx, mrmd_atoms* a, double dt, double* maxDisplacement)
{
    // action/VelocityVerlet.cpp:26-67
    if (!ctx || !a) return MRMD_ERR_ARG;
    double* dMax = ctx->devScalars + 24;
    MRMD_CUDA(ctx, cudaMemsetAsync(dMax, 0, sizeof(double), ctx->stream));
    const int64_t n = a->numLocal;
    if (n > 0)
    {
        k_vv_pre<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
            reinterpret_cast<double4*>(a->pos), reinterpret_cast<double4*>(a->vel),
            reinterpret_cast<const double4*>(a->force), a->mass, n, 0.5 * dt, dt, dMax);
        MRMD_TRY(after_launch(ctx, "vv_pre"));
    }
    return read_max_disp(ctx, dMax, maxDisplacement);
}

int mrmd_vv_post(mrmd_ctx* ctx, mrmd_atoms* a, double dt)
{
    // action/VelocityVerlet.cpp:69-90
    if (!ctx || !a) return MRMD_ERR_ARG;
    const int64_t n = a->numLocal;
    if (n > 0)
    {
        k_vv_post<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
            reinterpret_cast<double4*>(a->vel), reinterpret_cast<const double4*>(a->force), a->mass, n, 0.5 * dt);
        MRMD_TRY(after_launch(ctx, "vv_post"));
    }
    return finish(ctx, "vv_post");
}

int mrmd_langevin_pre(mrmd_ctx* ctx, mrmd_atoms* a, double dt, double zeta, double temperature, uint64_t seed,
                      uint64_t step, const mrmd_pred* pred, double* maxDisplacement)
{
    if (!ctx || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(pred_valid(pred), ctx, "bad predicate");
    double* dMax = ctx->devScalars + 24;
    MRMD_CUDA(ctx, cudaMemsetAsync(dMax, 0, sizeof(double), ctx->stream));
    const int64_t n = a->numLocal;
    if (n > 0)
    {
        k_langevin_pre<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
            reinterpret_cast<double4*>(a->pos), reinterpret_cast<double4*>(a->vel),
            reinterpret_cast<const double4*>(a->force), a->mass, n, 0.5 * dt, dt, zeta, temperature, seed, step,
            to_dev_pred(pred), dMax);
        MRMD_TRY(after_launch(ctx, "langevin_pre"));
    }
    return read_max_disp(ctx, dMax, maxDisplacement);
}

}  // extern "C"
