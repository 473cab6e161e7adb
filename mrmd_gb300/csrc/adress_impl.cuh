// AdResS device helpers shared by LJ_IdealGas, UpdateMolecules and the
// batched replica engine: the Slab weighting function, the region checks and
// the drift-compensation histogram bin.
#pragma once

#include <cmath>

#include "common.cuh"

namespace mrmd_impl
{
constexpr int COMP_BINS = 200;  // LJ_IdealGas.hpp:54

struct SlabDev
{
    double cx;
    double atHalf;  // atomisticRegionHalfDiameter
    double hy;      // hybridRegionDiameter
    int64_t exponent;
    int32_t abrupt;
};

__device__ __forceinline__ double pow_int(double x, int64_t n)
{
    // util/math.hpp:31-46
    double ww = x, yy = 1.0;
    for (int64_t nn = (n > 0) ? n : -n; nn != 0; nn >>= 1)
    {
        if ((nn & 1) == 1) yy *= ww;
        ww *= ww;
    }
    return (n > 0) ? yy : 1.0 / yy;
}

__device__ __forceinline__ void slab_eval(const SlabDev& s, double x, double& lambda, double& modLambda,
                                          double& gx)
{
    // weighting_function/Slab.hpp:161-187 (+ setSmoothWeightInHY :96-120)
    const double pi = 3.141592653589793238462643383279502884;
    const double dx = x - s.cx;
    const double absDx = fabs(dx);
    gx = 0.0;
    if (absDx < s.atHalf)
    {
        lambda = 1.0;
        modLambda = 1.0;
    }
    else if (absDx > s.atHalf + s.hy)
    {
        lambda = 0.0;
        modLambda = 0.0;
    }
    else if (s.abrupt)
    {
        lambda = 1.0;
        modLambda = 1.0;
    }
    else
    {
        const double arg = pi / (2.0 * s.hy) * (absDx - s.atHalf);
        const double base = cos(arg);
        lambda = base * base;
        modLambda = pow_int(base, s.exponent);
        const double factor =
            -pi / (2.0 * s.hy) * (double)s.exponent * sin(arg) * pow_int(base, s.exponent - 1) / absDx;
        gx = factor * dx;
    }
}

// CheckRegion.hpp:25-38 with REGION_CHECK_EPSILON = 0
__device__ __forceinline__ bool is_at(double l) { return l >= 1.0; }
__device__ __forceinline__ bool is_cg(double l) { return l <= 0.0; }
__device__ __forceinline__ bool is_hy(double l) { return !is_at(l) && !is_cg(l); }

__device__ __forceinline__ int comp_bin(double lambda)
{
    // MultiHistogram(0, 1, 200).getBin (data/MultiHistogram.hpp:60-66)
    const double inv = 1.0 / ((1.0 - 0.0) / (double)COMP_BINS);
    int64_t b = (int64_t)floor((lambda - 0.0) * inv);
    if (b < 0 || b >= COMP_BINS) return -1;
    return (int)b;
}

inline SlabDev to_slab(const mrmd_slab* s)
{
    // Slab constructor, weighting_function/Slab.hpp:189-200
    SlabDev d{};
    d.cx = s->center[0];
    d.atHalf = 0.5 * s->atomisticRegionDiameter;
    d.hy = s->hybridRegionDiameter;
    d.exponent = 2 * s->nu;
    d.abrupt = s->interfaceType == 1;
    return d;
}
}  // namespace mrmd_impl
