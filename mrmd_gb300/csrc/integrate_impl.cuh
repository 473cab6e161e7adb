// Per-atom integrator building blocks (action/UpdateSteps.hpp:25-79) and
// the counter-based normal generator that replaces the reference's
// Random_XorShift1024_Pool.
#pragma once

#include <cmath>

#include "common.cuh"

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

// Three standard normals for (seed, step, atom): Philox block -> four
// uniforms in (0,1) -> two Box-Muller pairs.
__device__ __forceinline__ void normal3(uint64_t seed, uint64_t step, uint64_t atom, double g[3])
{
    uint32_t c[4] = {(uint32_t)atom, (uint32_t)(atom >> 32), (uint32_t)step, (uint32_t)(step >> 32)};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double s = 2.3283064365386963e-10;  // 2^-32
    const double u0 = ((double)c[0] + 0.5) * s;
    const double u1 = ((double)c[1] + 0.5) * s;
    const double u2 = ((double)c[2] + 0.5) * s;
    const double u3 = ((double)c[3] + 0.5) * s;
    const double twoPi = 6.283185307179586;
    const double ra = sqrt(-2.0 * log(u0));
    const double rb = sqrt(-2.0 * log(u2));
    g[0] = ra * cos(twoPi * u1);
    g[1] = ra * sin(twoPi * u1);
    g[2] = rb * cos(twoPi * u3);
}

// updateOrnsteinUhlenbeck (UpdateSteps.hpp:56-79)
__device__ __forceinline__ void ornstein_uhlenbeck(double4& v, double dt, double m, double zeta, double T,
                                                   const double g[3])
{
    const double dtm = __ddiv_rn(dt, m);
    const double damping = exp(-zeta * dtm);
    const double sigma = sqrt(T / m * (1.0 - exp(-2.0 * zeta * dtm)));
    v.x = __dmul_rn(v.x, damping);
    v.y = __dmul_rn(v.y, damping);
    v.z = __dmul_rn(v.z, damping);
    v.x = __dadd_rn(v.x, __dmul_rn(sigma, g[0]));
    v.y = __dadd_rn(v.y, __dmul_rn(sigma, g[1]));
    v.z = __dadd_rn(v.z, __dmul_rn(sigma, g[2]));
}
}  // namespace mrmd_impl
