// action::ThermodynamicForce: x-density sampling (analysis::getAxialDensityProfile),
// table application (apply_if / applyInterpolated_if) and the table update
// (MultiHistogram makeSymmetric / scale / smoothen / gradient / replace_if).
//
// Sampling privatises the (bins x types) histogram in shared memory per
// block and adds each block's integer counts once, so the result is exact
// and independent of thread order.  The update runs the whole pipeline of
// ThermodynamicForce::update_if in one single-block launch (a few hundred
// bins), in the reference's per-bin arithmetic order.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "thermo_impl.cuh"

using namespace mrmd_impl;

struct mrmd_tf
{
    double min = 0, max = 0, binSize = 0, inverseBinSize = 0, binVolume = 0;
    int64_t numBins = 0, numTypes = 0, samples = 0;
    int enforceSymmetry = 0, usePeriodicity = 0;
    std::vector<double> forceFactor;
    double* dForce = nullptr;    // [numBins][numTypes]
    double* dDensity = nullptr;  // [numBins][numTypes]
    double* dWork = nullptr;     // 2 x [numBins][numTypes] + numTypes
};

namespace
{
constexpr int TB = 256;

__global__ void k_density(const double4* __restrict__ pos, const int32_t* __restrict__ type, int64_t n, HistDev h,
                          double* __restrict__ density, int useShared)
{
    // analysis/AxialDensityProfile.cpp:36-47
    extern __shared__ unsigned int sh[];
    const int64_t nbh = h.numBins * h.numTypes;
    if (useShared)
    {
        for (int64_t k = threadIdx.x; k < nbh; k += blockDim.x) sh[k] = 0u;
        __syncthreads();
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t b = get_bin(h, pos[i].x);
        if (b == -1) continue;
        const int64_t k = b * h.numTypes + type[i];
        if (useShared)
            atomicAdd(&sh[k], 1u);
        else
            atomicAdd(&density[k], 1.0);
    }
    if (useShared)
    {
        __syncthreads();
        for (int64_t k = threadIdx.x; k < nbh; k += blockDim.x)
            if (sh[k]) atomicAdd(&density[k], (double)sh[k]);
    }
}

__global__ void k_tf_apply(double4* __restrict__ force, const double4* __restrict__ pos,
                           const int32_t* __restrict__ type, int64_t n, HistDev h, const double* __restrict__ table,
                           mrmd_dev::Pred pred, int interpolated)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
    {
        const double4 p = pos[i];
        const double xPos = p.x;
        if (!mrmd_dev::pred1(pred, p.x, p.y, p.z)) continue;
        const int64_t bin = get_bin(h, xPos);
        if (bin == -1) continue;
        const int32_t t = type[i];
        double add;
        if (!interpolated)
        {
            // ThermodynamicForce.hpp:107-119
            add = table[bin * h.numTypes + t];
        }
        else
        {
            // ThermodynamicForce.hpp:163-213
            const double binStart = h.min + (double)bin * h.binSize;
            const double fracInBin = (xPos - binStart) * h.inverseBinSize;
            int64_t l, r;
            double factor;
            if (fracInBin < 0.5)
            {
                l = bin - 1;
                r = bin;
                factor = fracInBin + 0.5;
            }
            else
            {
                l = bin;
                r = bin + 1;
                factor = fracInBin - 0.5;
            }
            if (l >= 0 && r < h.numBins)
            {
                const double a = table[l * h.numTypes + t], b = table[r * h.numTypes + t];
                add = a + (b - a) * factor;  // util/interpolation.hpp:34-37
            }
            else
            {
                add = table[bin * h.numTypes + t];
            }
        }
        force[i].x = __dadd_rn(force[i].x, add);
    }
}

__global__ void k_tf_update(UpdateArgs A) { tf_update_block(A); }

HistDev hist_of(const mrmd_tf* tf)
{
    HistDev h{};
    h.min = tf->min;
    h.binSize = tf->binSize;
    h.inverseBinSize = tf->inverseBinSize;
    h.numBins = tf->numBins;
    h.numTypes = tf->numTypes;
    return h;
}
}  // namespace

extern "C" {

int mrmd_tf_create(mrmd_ctx* ctx, mrmd_tf** out, int64_t numTypes, const double* targetDensity,
                   const mrmd_subdomain* sd, double requestedBinWidth, const double* modulation, int enforceSymmetry,
                   int usePeriodicity)
{
    // action/ThermodynamicForce.cpp:25-57
    if (!ctx || !out || !targetDensity || !sd || !modulation) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(numTypes > 0, ctx, "numTypes must be > 0");
    MRMD_CHECK_ARG(requestedBinWidth > 0.0, ctx, "bin width must be > 0");
    *out = nullptr;
    mrmd_tf* tf = new mrmd_tf();
    tf->numTypes = numTypes;
    tf->numBins = (int64_t)std::ceil(sd->diameter[0] / requestedBinWidth);
    tf->min = sd->minCorner[0];
    tf->max = sd->maxCorner[0];
    tf->binSize = (tf->max - tf->min) / (double)tf->numBins;  // MultiHistogram.hpp:40-41
    tf->inverseBinSize = 1.0 / tf->binSize;
    if (!(tf->binSize <= requestedBinWidth))
    {
        delete tf;
        return set_error(ctx, MRMD_ERR_ARG, "requested bin size is not achieved");
    }
    tf->binVolume = sd->diameter[1] * sd->diameter[2] * tf->binSize;
    tf->enforceSymmetry = enforceSymmetry;
    tf->usePeriodicity = usePeriodicity;
    tf->forceFactor.resize((size_t)numTypes);
    for (int64_t t = 0; t < numTypes; ++t) tf->forceFactor[(size_t)t] = modulation[t] / targetDensity[t];
    const size_t nbh = (size_t)(tf->numBins * numTypes);
    int rc = dmalloc(ctx, reinterpret_cast<void**>(&tf->dForce), sizeof(double) * nbh);
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&tf->dDensity), sizeof(double) * nbh);
    if (rc == MRMD_OK) rc = dmalloc(ctx, reinterpret_cast<void**>(&tf->dWork), sizeof(double) * (2 * nbh + numTypes));
    if (rc == MRMD_OK) rc = dzero(ctx, tf->dForce, sizeof(double) * nbh);
    if (rc == MRMD_OK) rc = dzero(ctx, tf->dDensity, sizeof(double) * nbh);
    if (rc == MRMD_OK)
        rc = h2d(ctx, tf->dWork + 2 * nbh, tf->forceFactor.data(), sizeof(double) * numTypes);
    if (rc != MRMD_OK)
    {
        dfree(tf->dForce);
        dfree(tf->dDensity);
        dfree(tf->dWork);
        delete tf;
        return rc;
    }
    *out = tf;
    return MRMD_OK;
}

int mrmd_tf_destroy(mrmd_ctx* ctx, mrmd_tf* tf)
{
    if (!tf) return MRMD_OK;
    if (ctx) cudaStreamSynchronize(ctx->stream);
    dfree(tf->dForce);
    dfree(tf->dDensity);
    dfree(tf->dWork);
    delete tf;
    return MRMD_OK;
}

int mrmd_tf_shape(const mrmd_tf* tf, int64_t* numBins, double* binSize, int64_t* numTypes)
{
    if (!tf) return MRMD_ERR_ARG;
    if (numBins) *numBins = tf->numBins;
    if (binSize) *binSize = tf->binSize;
    if (numTypes) *numTypes = tf->numTypes;
    return MRMD_OK;
}

int mrmd_tf_grid(const mrmd_tf* tf, double* grid)
{
    // data/MultiHistogram.cpp:214-227 with getBinPosition (MultiHistogram.hpp:68-74)
    if (!tf || !grid) return MRMD_ERR_ARG;
    for (int64_t i = 0; i < tf->numBins; ++i) grid[i] = tf->min + ((double)i + 0.5) * tf->binSize;
    return MRMD_OK;
}

int mrmd_tf_sample(mrmd_ctx* ctx, mrmd_tf* tf, const mrmd_atoms* a)
{
    // ThermodynamicForce.cpp:74-86
    if (!ctx || !tf || !a) return MRMD_ERR_ARG;
    const int64_t n = a->numLocal;
    if (n > 0)
    {
        const int64_t nbh = tf->numBins * tf->numTypes;
        const size_t smem = sizeof(unsigned int) * (size_t)nbh;
        const int useShared = smem <= 48 * 1024;
        k_density<<<grid_for(ctx, n, TB, 2), TB, useShared ? smem : 0, ctx->stream>>>(
            reinterpret_cast<const double4*>(a->pos), a->type, n, hist_of(tf), tf->dDensity, useShared);
        MRMD_TRY(after_launch(ctx, "tf_sample"));
    }
    tf->samples++;
    return finish(ctx, "tf_sample");
}

int mrmd_tf_apply(mrmd_ctx* ctx, const mrmd_tf* tf, mrmd_atoms* a, const mrmd_pred* pred, int interpolated)
{
    if (!ctx || !tf || !a) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(pred_valid(pred), ctx, "bad predicate");
    const int64_t n = a->numLocal;
    if (n == 0) return MRMD_OK;
    k_tf_apply<<<grid_for(ctx, n, TB), TB, 0, ctx->stream>>>(reinterpret_cast<double4*>(a->force),
                                                              reinterpret_cast<const double4*>(a->pos), a->type, n,
                                                              hist_of(tf), tf->dForce, to_dev_pred(pred),
                                                              interpolated ? 1 : 0);
    MRMD_TRY(after_launch(ctx, "tf_apply"));
    return finish(ctx, "tf_apply");
}

int mrmd_tf_update(mrmd_ctx* ctx, mrmd_tf* tf, double smoothingSigma, double smoothingIntensity,
                   const mrmd_pred* pred)
{
    if (!ctx || !tf) return MRMD_ERR_ARG;
    MRMD_CHECK_ARG(pred_valid(pred), ctx, "bad predicate");
    if (tf->samples <= 0) return set_error(ctx, MRMD_ERR_STATE, "no density samples (ThermodynamicForce.hpp:129)");
    const int64_t nbh = tf->numBins * tf->numTypes;
    UpdateArgs A{};
    A.density = tf->dDensity;
    A.force = tf->dForce;
    A.smooth = tf->dWork;
    A.grad = tf->dWork + nbh;
    A.forceFactor = tf->dWork + 2 * nbh;
    A.numBins = tf->numBins;
    A.numTypes = tf->numTypes;
    A.binSize = tf->binSize;
    A.inverseBinSize = tf->inverseBinSize;
    A.min = tf->min;
    A.normalization = 1.0 / (tf->binVolume * (double)tf->samples);
    A.sigma = smoothingSigma;
    A.range = smoothingIntensity;
    A.enforceSymmetry = tf->enforceSymmetry;
    A.periodic = tf->usePeriodicity;
    A.pred = to_dev_pred(pred);
    A.usePred = pred != nullptr;
    k_tf_update<<<1, 1024, 0, ctx->stream>>>(A);
    MRMD_TRY(after_launch(ctx, "tf_update"));
    tf->samples = 0;
    return finish(ctx, "tf_update");
}

int mrmd_tf_get_force(mrmd_ctx* ctx, const mrmd_tf* tf, double* out)
{
    if (!ctx || !tf || !out) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MRMD_TRY(d2h(ctx, out, tf->dForce, sizeof(double) * (size_t)(tf->numBins * tf->numTypes)));
    return MRMD_OK;
}

int mrmd_tf_set_force(mrmd_ctx* ctx, mrmd_tf* tf, const double* in)
{
    if (!ctx || !tf || !in) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MRMD_TRY(h2d(ctx, tf->dForce, in, sizeof(double) * (size_t)(tf->numBins * tf->numTypes)));
    return MRMD_OK;
}

int mrmd_tf_get_density(mrmd_ctx* ctx, const mrmd_tf* tf, double* out, int64_t* samples)
{
    if (!ctx || !tf) return MRMD_ERR_ARG;
    MRMD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (out)
        MRMD_TRY(d2h(ctx, out, tf->dDensity, sizeof(double) * (size_t)(tf->numBins * tf->numTypes)));
    if (samples) *samples = tf->samples;
    return MRMD_OK;
}

int mrmd_tf_mu(mrmd_ctx* ctx, const mrmd_tf* tf, double* muLeft, double* muRight)
{
    // ThermodynamicForce.cpp:98-130 (host reduction of the table, as the reference)
    if (!ctx || !tf || !muLeft || !muRight) return MRMD_ERR_ARG;
    std::vector<double> F((size_t)(tf->numBins * tf->numTypes));
    MRMD_TRY(mrmd_tf_get_force(ctx, tf, F.data()));
    for (int64_t t = 0; t < tf->numTypes; ++t)
    {
        double l = 0.0, r = 0.0;
        for (int64_t i = 0; i < tf->numBins / 2; ++i) l += F[(size_t)(i * tf->numTypes + t)];
        for (int64_t i = tf->numBins / 2; i < tf->numBins; ++i) r += F[(size_t)(i * tf->numTypes + t)];
        muLeft[t] = l * tf->binSize;
        muRight[t] = r * tf->binSize;
    }
    return MRMD_OK;
}

}  // extern "C"
