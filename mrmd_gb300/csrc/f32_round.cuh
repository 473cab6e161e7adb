// FP64 -> FP32 round-to-nearest-even with integer operations only.  GB300
// runs FP64 conversions on its small FP64 pipe (2 operations per clock per
// SM); kernels that are bound by that pipe convert with these instead.
// Host and device (the host form is tested against the C cast).
#pragma once

#include <cmath>
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

__host__ __device__ inline uint32_t f32_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t b;
    std::memcpy(&b, &f, sizeof(b));
    return b;
#endif
}

__host__ __device__ inline double f64_from_bits(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
#endif
}

// The double of a float (exact, subnormals and NaN payloads included), with
// integer operations only.
__host__ __device__ inline double f32_to_f64(float f)
{
    const uint32_t b = f32_bits(f);
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint32_t e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    uint64_t bits;
    if (e == 0xffu)
        bits = 0x7ff0000000000000ull | ((uint64_t)m << 29);
    else if (e != 0)
        bits = ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
    else if (m == 0)
        bits = 0;
    else
    {
        // subnormal: m 2^-149 with the leading one of m at bit p
#ifdef __CUDA_ARCH__
        const int p = 31 - __clz((int)m);
#else
        const int p = 31 - __builtin_clz(m);
#endif
        bits = ((uint64_t)(p + 874) << 52) | ((uint64_t)(m ^ (1u << p)) << (52 - p));
    }
    return f64_from_bits(sign | bits);
}

// The float nearest to r 2^E (ties to even), r a signed integer, with
// integer operations only.
__host__ __device__ inline float scaled_i64_to_f32_rn(int64_t r, int E)
{
    if (r == 0) return 0.0f;
    const uint32_t sign = r < 0 ? 0x80000000u : 0u;
    const uint64_t a = r < 0 ? (uint64_t)0 - (uint64_t)r : (uint64_t)r;
#ifdef __CUDA_ARCH__
    const int p = 63 - __clzll((long long)a);
#else
    const int p = 63 - __builtin_clzll(a);
#endif
    const int be = p + E + 127;  // biased float exponent of r 2^E (normal case)
    uint32_t bits;
    if (be >= 255)
        bits = 0x7f800000u;
    else if (be >= 1)
    {
        uint64_t m;
        if (p > 23)
        {
            const int s = p - 23;
            m = a >> s;
            const uint64_t rest = a & ((1ull << s) - 1ull), half = 1ull << (s - 1);
            m += (rest > half || (rest == half && (m & 1ull))) ? 1ull : 0ull;
        }
        else
            m = a << (23 - p);
        // m in [2^23, 2^24]: its leading one adds one to the exponent field
        // (a rounding carry to 2^24 adds two and clears the fraction)
        bits = ((uint32_t)(be - 1) << 23) + (uint32_t)m;
        if (bits >= 0x7f800000u) bits = 0x7f800000u;
    }
    else
    {
        // subnormal float: units of 2^-149
        const int s = -(E + 149);
        uint64_t q;
        if (s <= 0)
            q = a << (-s);  // below 2^23 here
        else if (s >= 64)
            q = 0;
        else
        {
            q = a >> s;
            const uint64_t rest = a & ((1ull << s) - 1ull), half = 1ull << (s - 1);
            q += (rest > half || (rest == half && (q & 1ull))) ? 1ull : 0ull;
        }
        bits = (uint32_t)q;
    }
    return f32_from_bits(sign | bits);
}

// The coordinate split hi = k Q, lo = x - o - k Q rounded to FP32, with
// k the integer nearest to (x - o) / Q (ties to even k), Q = 2^-q and the
// origin o = Ko Q, from the bits of x with integer operations only.  For
// finite x with |x / Q| < 2^61 and |k| < 2^24 it gives, bit for bit, what
// the three FP64 additions of the magic-number form give (t = x + (magic -
// o) rounds to the Q grid with ties to the even significand, that is, to
// even k).
__host__ __device__ inline void split_bits(double x, long long Ko, int q, float invScaleF, float& h, float& l)
{
    const uint64_t b = f64_bits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    const int64_t M = (int64_t)((b & 0xfffffffffffffull) | (e ? (1ull << 52) : 0ull));
    const int E = (e ? e : 1) - 1075;  // x = X 2^E
    const int64_t X = (b >> 63) ? -M : M;
    const int sh = -(E + q);  // fractional bits of x / Q in X
    int64_t kx, r;            // x / Q = kx + r 2^-sh
    if (sh <= 0)
    {
        // x a multiple of Q (a non-finite x, reported by the next rebuild's
        // binning, lands here too: no shift of 62 bits or more)
        kx = -sh < 62 ? (int64_t)((uint64_t)X << (-sh)) : 0;
        r = 0;
    }
    else if (sh >= 62)
    {
        kx = 0;  // |x / Q| < 2^-9
        r = X;
    }
    else
    {
        const int64_t fl = X >> sh;  // floor (arithmetic shift)
        const int64_t fr = X - (int64_t)((uint64_t)fl << sh);
        const int64_t half = (int64_t)1 << (sh - 1);
        const bool up = fr > half || (fr == half && ((fl - Ko) & 1));
        kx = up ? fl + 1 : fl;
        r = up ? fr - ((int64_t)1 << sh) : fr;
    }
    const int32_t k = (int32_t)(kx - Ko);
#ifdef __CUDA_ARCH__
    h = __fmul_rn(__int2float_rn(k), invScaleF);
#else
    h = (float)k * invScaleF;
#endif
    l = scaled_i64_to_f32_rn(r, E);
}

#ifdef __CUDA_ARCH__
#define MRMD_FADD(a, b) __fadd_rn(a, b)
#define MRMD_FSUB(a, b) __fsub_rn(a, b)
#define MRMD_FMUL(a, b) __fmul_rn(a, b)
#else
#define MRMD_FADD(a, b) ((float)(a) + (float)(b))
#define MRMD_FSUB(a, b) ((float)(a) - (float)(b))
#define MRMD_FMUL(a, b) ((float)(a) * (float)(b))
#endif

// floor(fl(fl(x - mn) * rdx)) (FP64 operations) from an FP32 estimate, when
// the estimate's error interval holds no integer: *ok false otherwise
// (and for NaN / infinite / huge x), where the caller evaluates the FP64
// formula.  mnf, rdxf: mn and rdx rounded to FP32.  The estimate's error is
// below (|x| + |mn| + 3 |x - mn|) rdx 2^-24 (the roundings of x, mn, rdx,
// the difference and the product; the FP64 value's own error is ~2^-52
// relative); the interval is four times that.
__host__ __device__ inline float floor_of_scaled(double x, float mnf, float rdxf, bool* ok)
{
    const float xf = f64_to_f32_rn(x);
    const float d = MRMD_FSUB(xf, mnf);
    const float tf = MRMD_FMUL(d, rdxf);
    const float ax = xf < 0.f ? -xf : xf, am = mnf < 0.f ? -mnf : mnf, ad = d < 0.f ? -d : d;
    const float at = tf < 0.f ? -tf : tf;
    const float err = MRMD_FMUL(MRMD_FADD(MRMD_FMUL(MRMD_FADD(MRMD_FADD(ax, am), MRMD_FADD(ad, ad)), rdxf), at),
                                2.384185791015625e-7f);  // 2^-22
    const float lo = std::floor(MRMD_FSUB(tf, err)), hi = std::floor(MRMD_FADD(tf, err));
    *ok = lo == hi;  // false for NaN
    return lo;
}
}  // namespace mrmd_impl
