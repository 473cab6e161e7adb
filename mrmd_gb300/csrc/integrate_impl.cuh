// Per-atom integrator building blocks (action/UpdateSteps.hpp:25-79) and
// the counter-based normal generator that replaces the reference's
// Random_XorShift1024_Pool.
#pragma once

#include <cmath>

#include "common.cuh"
#include "f32_round.cuh"

namespace mrmd_impl
{
// updateKick: v += (dt/m) * F   (UpdateSteps.hpp:25-39), dtfm precomputed
__device__ __forceinline__ void kick(double4& v, const double4& f, double dtfm)
{
    v.x = __dadd_rn(v.x, __dmul_rn(dtfm, f.x));
    v.y = __dadd_rn(v.y, __dmul_rn(dtfm, f.y));
    v.z = __dadd_rn(v.z, __dmul_rn(dtfm, f.z));
}

// updateDrift: x += dt * v   (UpdateSteps.hpp:41-54)
__device__ __forceinline__ void drift(double4& x, const double4& v, double dt)
{
    x.x = __dadd_rn(x.x, __dmul_rn(dt, v.x));
    x.y = __dadd_rn(x.y, __dmul_rn(dt, v.y));
    x.z = __dadd_rn(x.z, __dmul_rn(dt, v.z));
}

// The same updates with one rounding each (fused multiply-add).
__device__ __forceinline__ void kick_fma(double4& v, const double4& f, double dtfm)
{
    v.x = __fma_rn(dtfm, f.x, v.x);
    v.y = __fma_rn(dtfm, f.y, v.y);
    v.z = __fma_rn(dtfm, f.z, v.z);
}

// 2 d, exactly, on the integer pipe (d finite and not negative zero)
__device__ __forceinline__ double twice(double d)
{
    const long long b = __double_as_longlong(d);
    const long long e = b & 0x7ff0000000000000ll;
    return __longlong_as_double(b + (e ? (1ll << 52) : (b & 0x000fffffffffffffll)));
}

__device__ __forceinline__ void drift_fma(double4& x, const double4& v, double dt)
{
    x.x = __fma_rn(dt, v.x, x.x);
    x.y = __fma_rn(dt, v.y, x.y);
    x.z = __fma_rn(dt, v.z, x.z);
}

// util::dot3 of (x0 - x)   (VelocityVerlet.cpp:55-59)
__device__ __forceinline__ double disp_sqr(const double4& x0, const double4& x)
{
    const double dx = __dsub_rn(x0.x, x.x), dy = __dsub_rn(x0.y, x.y), dz = __dsub_rn(x0.z, x.z);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// VelocityVerlet::preForceIntegrate body for one atom; returns |dx|^2.
__device__ __forceinline__ double vv_pre_one(double4 x, double4 v, const double4& f, double m, double dtHalf,
                                             double dt, double4* xOut, double4* vOut)
{
    const double4 x0 = x;
    kick(v, f, __ddiv_rn(dtHalf, m));
    drift(x, v, dt);
    *xOut = x;
    *vOut = v;
    return disp_sqr(x0, x);
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r)
    {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
        const uint32_t lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
        const uint32_t lo1 = 0xCD9E8D57u * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0;
        const uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Standard normals from a Philox block by Box-Muller in FP32 (the thermostat
// needs statistics, not digits).  ln and sin/cos are our own: a reduction to
// a mantissa in [sqrt(1/2), sqrt(2)] with the series 2 atanh(t), t = (m-1)/(m+1),
// and a quarter-turn reduction of the angle with Taylor polynomials on
// [-pi/4, pi/4].  Every operation is a correctly rounded FP32 add, multiply,
// divide, square root or FMA, so the host restatement computes the same bits.
__device__ __forceinline__ float bm_log(float u)  // u in (0, 1)
{
    const int bits = __float_as_int(u);
    int e = ((bits >> 23) & 0xff) - 127;
    float m = __int_as_float((bits & 0x7fffff) | 0x3f800000);  // [1, 2)
    if (m > 0x1.6a09e6p+0f)
    {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float t = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float t2 = __fmul_rn(t, t);
    float p = __fmaf_rn(t2, 0x1.c71c72p-4f, 0x1.24924ap-3f);  // 1/9, 1/7
    p = __fmaf_rn(p, t2, 0x1.99999ap-3f);                      // 1/5
    p = __fmaf_rn(p, t2, 0x1.555556p-2f);                      // 1/3
    p = __fmaf_rn(p, t2, 1.0f);
    return __fmaf_rn((float)e, 0x1.62e430p-1f, __fmul_rn(2.0f, __fmul_rn(t, p)));  // e ln2 + 2 atanh(t)
}

// cos and sin of 2 pi u, u in (0, 1)
__device__ __forceinline__ void bm_sincos(float u, float& c, float& s)
{
    const float q = rintf(__fmul_rn(4.0f, u));
    const float x = __fsub_rn(u, __fmul_rn(0.25f, q));  // exact, |x| <= 1/8
    const float f = __fmul_rn(x, 0x1.921fb6p+2f);        // 2 pi x, |f| <= pi/4
    const float f2 = __fmul_rn(f, f);
    float ps = __fmaf_rn(f2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    ps = __fmaf_rn(ps, f2, 0x1.111112p-7f);
    ps = __fmaf_rn(ps, f2, -0x1.555556p-3f);
    const float sn = __fmaf_rn(__fmul_rn(f, f2), ps, f);
    float pc = __fmaf_rn(f2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    pc = __fmaf_rn(pc, f2, -0x1.6c16c2p-10f);
    pc = __fmaf_rn(pc, f2, 0x1.555556p-5f);
    pc = __fmaf_rn(pc, f2, -0.5f);
    const float cs = __fmaf_rn(pc, f2, 1.0f);
    const int quadrant = ((int)q) & 3;  // angle = f + quadrant * pi/2
    c = quadrant == 0 ? cs : (quadrant == 1 ? -sn : (quadrant == 2 ? -cs : sn));
    s = quadrant == 0 ? sn : (quadrant == 1 ? cs : (quadrant == 2 ? -sn : -cs));
}

// Three standard normals for (seed, step, atom): one Philox block -> four
// 23-bit uniforms in (0, 1) -> two Box-Muller pairs (the third value of the
// second pair is unused).
__device__ __forceinline__ void normal3(uint64_t seed, uint64_t step, uint64_t atom, double g[3])
{
    uint32_t c[4] = {(uint32_t)atom, (uint32_t)(atom >> 32), (uint32_t)step, (uint32_t)(step >> 32)};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    float u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = __fmul_rn(__fadd_rn((float)(c[k] >> 9), 0.5f), 0x1p-23f);
    const float ra = __fsqrt_rn(__fmul_rn(-2.0f, bm_log(u[0])));
    const float rb = __fsqrt_rn(__fmul_rn(-2.0f, bm_log(u[2])));
    float ca, sa, cb, sb;
    bm_sincos(u[1], ca, sa);
    bm_sincos(u[3], cb, sb);
    // exact widening on the integer pipe (the FP64 pipe bounds the kernels
    // that draw the noise)
    g[0] = f32_to_f64(__fmul_rn(ra, ca));
    g[1] = f32_to_f64(__fmul_rn(ra, sa));
    g[2] = f32_to_f64(__fmul_rn(rb, cb));
}

// Ornstein-Uhlenbeck coefficients of one mass (UpdateSteps.hpp:56-79):
// damping = exp(-zeta dt / m), sigma = sqrt(T / m (1 - exp(-2 zeta dt / m))).
struct OUCoef
{
    double m = -1.0, damping = 0.0, sigma = 0.0;

    __device__ __forceinline__ void update(double mass, double dt, double zeta, double T)
    {
        if (mass == m) return;  // uniform masses: computed once per thread
        const double dtm = __ddiv_rn(dt, mass);
        damping = exp(-zeta * dtm);
        sigma = sqrt(T / mass * (1.0 - exp(-2.0 * zeta * dtm)));
        m = mass;
    }
};

__device__ __forceinline__ void ornstein_uhlenbeck(double4& v, const OUCoef& k, const double g[3])
{
    v.x = __dmul_rn(v.x, k.damping);
    v.y = __dmul_rn(v.y, k.damping);
    v.z = __dmul_rn(v.z, k.damping);
    v.x = __dadd_rn(v.x, __dmul_rn(k.sigma, g[0]));
    v.y = __dadd_rn(v.y, __dmul_rn(k.sigma, g[1]));
    v.z = __dadd_rn(v.z, __dmul_rn(k.sigma, g[2]));
}

}  // namespace mrmd_impl
