// FP64 -> FP32 round-to-nearest-even with integer operations only.  GB300
// runs FP64 conversions on its small FP64 pipe (2 operations per clock per
// SM); kernels that are bound by that pipe convert with these instead.
// Host and device (the host form is tested against the C cast).
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace mrmd_impl
{
__host__ __device__ inline uint64_t f64_bits(double d)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, sizeof(b));
    return b;
#endif
}

__host__ __device__ inline float f32_from_bits(uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof(f));
    return f;
#endif
}

// The float nearest to d (ties to even), as the IEEE conversion gives it:
// subnormal results, overflow to infinity, NaN kept as a quiet NaN.
__host__ __device__ inline float f64_to_f32_rn(double d)
{
    const uint64_t b = f64_bits(d);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    const uint64_t frac = b & 0xfffffffffffffull;
    uint32_t bits;
    if (e == 0x7ff)
        bits = frac ? 0x7fc00000u | (uint32_t)(frac >> 29) : 0x7f800000u;
    else if (e >= 1023 + 128)
        bits = 0x7f800000u;  // at least 2^128: infinity
    else if (e > 896)
    {
        // normal float: exponent e - 1023 + 127, 23 of the 52 fraction bits;
        // a carry out of the fraction moves into the exponent (up to infinity)
        uint32_t m = (uint32_t)(frac >> 29);
        const uint32_t rest = (uint32_t)frac & 0x1fffffffu;
        m += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
        bits = ((uint32_t)(e - 896) << 23) + m;
    }
    else if (e == 0)
        bits = 0;  // zero or FP64 subnormal: below half the least float
    else
    {
        // subnormal float (or zero): units of 2^-149
        const int shift = 926 - e;  // >= 30
        if (shift >= 54)
            bits = 0;
        else
        {
            const uint64_t full = frac | (1ull << 52);
            uint64_t q = full >> shift;
            const uint64_t rest = full & ((1ull << shift) - 1ull), half = 1ull << (shift - 1);
            q += (rest > half || (rest == half && (q & 1ull))) ? 1ull : 0ull;
            bits = (uint32_t)q;
        }
    }
    return f32_from_bits(sign | bits);
}
}  // namespace mrmd_impl
