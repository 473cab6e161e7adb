// ThermodynamicForce device helpers shared by the single-system actions and
// the batched replica engine: the MultiHistogram bin rule and the table
// update pipeline (makeSymmetric, scale, smoothen, gradient, replace_if).
#pragma once

#include <cmath>

#include "common.cuh"

namespace mrmd_impl
{
struct HistDev
{
    double min, binSize, inverseBinSize;
    int64_t numBins, numTypes;
};

__device__ __forceinline__ int64_t get_bin(const HistDev& h, double v)
{
    // data/MultiHistogram.hpp:60-66
    int64_t b = (int64_t)floor((v - h.min) * h.inverseBinSize);
    if (b < 0) b = -1;
    if (b >= h.numBins) b = -1;
    return b;
}

struct UpdateArgs
{
    double* density;
    double* force;
    double* smooth;
    double* grad;
    const double* forceFactor;
    int64_t numBins, numTypes;
    double binSize, inverseBinSize, min;
    double normalization;
    double sigma, range;
    int enforceSymmetry, periodic;
    mrmd_dev::Pred pred;
    int usePred;
};

// ThermodynamicForce::update_if (ThermodynamicForce.hpp:124-152) on one
// (bins x types) table, run by one thread block.
__device__ __forceinline__ void tf_update_block(const UpdateArgs& A)
{
    const int64_t nb = A.numBins, nh = A.numTypes, nbh = nb * nh;
    double* d = A.density;
    if (A.enforceSymmetry)
    {
        // MultiHistogram.cpp:76-90
        const int64_t maxIdx = nb - 1;
        for (int64_t k = threadIdx.x; k < (nb / 2) * nh; k += blockDim.x)
        {
            const int64_t i = k / nh, j = k % nh;
            const double val = 0.5 * (d[i * nh + j] + d[(maxIdx - i) * nh + j]);
            d[i * nh + j] = val;
            d[(maxIdx - i) * nh + j] = val;
        }
        __syncthreads();
    }
    for (int64_t k = threadIdx.x; k < nbh; k += blockDim.x) d[k] = __dmul_rn(d[k], A.normalization);
    __syncthreads();
    // smoothen, MultiHistogram.cpp:163-212
    const double inverseSigma = 1.0 / A.sigma;
    const int64_t delta = (int64_t)(int)(A.range * A.sigma * A.inverseBinSize);
    for (int64_t k = threadIdx.x; k < nbh; k += blockDim.x)
    {
        const int64_t b = k / nh, h = k % nh;
        double normalization = 0.0, acc = 0.0;
        int64_t jMin = b - delta, jMax = b + delta;
        if (!A.periodic)
        {
            jMin = jMin < 0 ? 0 : jMin;
            jMax = jMax > nb - 1 ? nb - 1 : jMax;
        }
        for (int64_t j = jMin; j <= jMax; ++j)
        {
            int64_t m = j;
            if (A.periodic)
            {
                // MultiHistogram.cpp:190-195 maps once (+-numBins); a smoothing
                // range wider than the table needs the full modulo, which equals
                // that mapping whenever it stays inside the table
                m %= nb;
                if (m < 0) m += nb;
            }
            const double t = __dmul_rn(__dmul_rn((double)(b - j), A.binSize), inverseSigma);
            const double eFunc = exp(-__dmul_rn(t, t));
            normalization = __dadd_rn(normalization, eFunc);
            acc = __dadd_rn(acc, __dmul_rn(d[m * nh + h], eFunc));
        }
        A.smooth[k] = __ddiv_rn(acc, normalization);
    }
    __syncthreads();
    // gradient, MultiHistogram.cpp:113-161; scale by forceFactor; replace_if; force -= grad
    const double inv = A.inverseBinSize, inv2 = 0.5 * A.inverseBinSize;
    const double* s = A.smooth;
    for (int64_t k = threadIdx.x; k < nbh; k += blockDim.x)
    {
        const int64_t i = k / nh, j = k % nh;
        double g;
        if (nb == 1)
            g = 0.0;  // no neighbouring bin (the reference would index outside the table)
        else if (i == 0)
            g = A.periodic ? __dmul_rn(__dsub_rn(s[(i + 1) * nh + j], s[(nb - 1) * nh + j]), inv2)
                           : __dmul_rn(__dsub_rn(s[(i + 1) * nh + j], s[i * nh + j]), inv);
        else if (i == nb - 1)
            g = A.periodic ? __dmul_rn(__dsub_rn(s[j], s[(i - 1) * nh + j]), inv2)
                           : __dmul_rn(__dsub_rn(s[i * nh + j], s[(i - 1) * nh + j]), inv);
        else
            g = __dmul_rn(__dsub_rn(s[(i + 1) * nh + j], s[(i - 1) * nh + j]), inv2);
        g = __dmul_rn(g, A.forceFactor[j]);
        if (A.usePred)
        {
            const double x = A.min + ((double)i + 0.5) * A.binSize;  // getBinPosition
            if (!mrmd_dev::pred_coord(A.pred, x)) g = 0.0;
        }
        A.grad[k] = g;
    }
    __syncthreads();
    for (int64_t k = threadIdx.x; k < nbh; k += blockDim.x)
    {
        A.force[k] = __dsub_rn(A.force[k], A.grad[k]);
        d[k] = 0.0;
    }
}
}  // namespace mrmd_impl
