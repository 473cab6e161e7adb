// Lennard-Jones internals shared by the pair kernels, LJ_IdealGas and the
// fused stepper.
#pragma once

#include <vector>

#include "common.cuh"

namespace mrmd_impl
{
// Device copy of one type pair's PrecomputedValues plus double-float (hi, lo)
// splits of the factors for the mixed form.
struct LJDev
{
    double ff1, ff2, ef1, ef2;
    double rcSqr, capSqr, capDist, capCoeff, shift, eCap;
    float ff1h, ff1l, ff2h, ff2l;  // ff1 = ff1h + ff1l exactly to ~2^-48
    float ef1f, ef2f, shiftf, rcSqrf;
    float capSqrf, capCoeff_f, eCapf, capDistf;
    float capCoeff_l;  // capCoeff = capCoeff_f + capCoeff_l to ~2^-48
    // low parts of the energy factors (double-float energies of the mixed form)
    float ef1l, ef2l, shiftl, capDistl;
    float eCapShh, eCapShl;  // E(r_cap) - shift
};

inline LJDev to_dev(const mrmd_lj_params& p)
{
    LJDev d{};
    d.ff1 = p.ff1;
    d.ff2 = p.ff2;
    d.ef1 = p.ef1;
    d.ef2 = p.ef2;
    d.rcSqr = p.rcSqr;
    d.capSqr = p.cappingDistanceSqr;
    d.capDist = p.cappingDistance;
    d.capCoeff = p.cappingCoeff;
    d.shift = p.shift;
    d.eCap = p.energyAtCappingPoint;
    d.ff1h = (float)p.ff1;
    d.ff1l = (float)(p.ff1 - (double)d.ff1h);
    d.ff2h = (float)p.ff2;
    d.ff2l = (float)(p.ff2 - (double)d.ff2h);
    d.ef1f = (float)p.ef1;
    d.ef2f = (float)p.ef2;
    d.shiftf = (float)p.shift;
    d.rcSqrf = (float)p.rcSqr;
    d.capSqrf = (float)p.cappingDistanceSqr;
    d.capCoeff_f = (float)p.cappingCoeff;
    d.eCapf = (float)p.energyAtCappingPoint;
    d.capDistf = (float)p.cappingDistance;
    // low parts: each (hi, lo) pair holds the double to ~2^-48
    d.capCoeff_l = (float)(p.cappingCoeff - (double)d.capCoeff_f);
    d.ef1l = (float)(p.ef1 - (double)d.ef1f);
    d.ef2l = (float)(p.ef2 - (double)d.ef2f);
    d.shiftl = (float)(p.shift - (double)d.shiftf);
    d.capDistl = (float)(p.cappingDistance - (double)d.capDistf);
    const double ecs = p.energyAtCappingPoint - p.shift;
    d.eCapShh = (float)ecs;
    d.eCapShl = (float)(ecs - (double)d.eCapShh);
    return d;
}

// computeForceAndEnergy (action/LennardJones.hpp:52-78) in FP64; the
// reciprocal is the correctly rounded one, identical to 1.0 / distSqr.
// The reference's formulae with every rounding explicit (fused
// multiply-adds where a product meets a sum, nothing left to the compiler's
// contraction): the same bits in every kernel that inlines it.
__device__ __forceinline__ void lj_eval_fp64(const LJDev& p, double distSqr, double& ff, double& e)
{
    if (distSqr >= p.capSqr)
    {
        const double frac2 = __drcp_rn(distSqr);
        const double frac6 = __dmul_rn(__dmul_rn(frac2, frac2), frac2);
        ff = __dmul_rn(__dmul_rn(frac6, __fma_rn(p.ff1, frac6, -p.ff2)), frac2);
        e = __fma_rn(frac6, __fma_rn(p.ef1, frac6, -p.ef2), -p.shift);
        return;
    }
    const double dist = __dsqrt_rn(distSqr);
    ff = __ddiv_rn(p.capCoeff, dist);
    e = __dsub_rn(__fma_rn(-__dsub_rn(dist, p.capDist), p.capCoeff, p.eCap), p.shift);
}

void lj_force_energy_host(const mrmd_lj_params* t, double distSqr, int64_t typeIdx, double* ff, double* e);
void lj_table_host(mrmd_lj_params* out, int64_t numTypes, const double* cap, const double* rc,
                   const double* sigma, const double* epsilon, int isShifted);

// ------------------------------------------------- double-float helpers --
// Error-free transformations (Knuth TwoSum, Dekker/FMA TwoProd); the pair
// (hi, lo) represents hi + lo with |lo| <= ulp(hi)/2 after renormalisation.
struct df
{
    float h, l;
};

__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ df df_mul(df a, df b)
{
    const float p = a.h * b.h;
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ df df_sqr(df a)
{
    const float p = a.h * a.h;
    float e = __fmaf_rn(a.h, a.h, -p);
    e = __fmaf_rn(2.0f * a.h, a.l, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ df df_add(df a, df b)
{
    df s = two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return fast_two_sum(s.h, s.l);
}

// 1/a with one Newton step on the double-float residual.  The seed is the
// hardware's approximate reciprocal (a correctly rounded one would cost a
// multi-instruction sequence and gains nothing: the Newton step squares
// the seed's ~2^-23 error).
__device__ __forceinline__ df df_rcp(df a)
{
    const float y = __fdividef(1.0f, a.h);
    float r = __fmaf_rn(-a.h, y, 1.0f);
    r = __fmaf_rn(-a.l, y, r);
    return fast_two_sum(y, y * r);
}

// sqrt(a) from the approximate reciprocal square root and one Newton
// correction on the exact FMA residual (a > 0)
__device__ __forceinline__ df df_sqrt(df a)
{
    const float q = rsqrtf(a.h);
    const float s = a.h * q;
    const float r = __fmaf_rn(-s, s, a.h) + a.l;
    return fast_two_sum(s, r * (0.5f * q));
}

// compensated accumulator (TwoSum), ~2^-48 relative to the final sum
__device__ __forceinline__ void df_acc(df& s, float x)
{
    const df t = two_sum(s.h, x);
    s.h = t.h;
    s.l += t.l;
}

}  // namespace mrmd_impl

struct mrmd_lj
{
    int64_t numTypes = 1;
    int64_t numTypesIndex = 1;
    double rcSqr = 0.0;
    std::vector<mrmd_lj_params> table;
    mrmd_impl::LJDev p0{};
    mrmd_impl::LJDev* dTable = nullptr;
};

namespace mrmd_impl
{
int lj_apply_fp64(mrmd_ctx* ctx, const mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl,
                  const mrmd_pred* pred, double* ev);
int lj_apply_mixed(mrmd_ctx* ctx, const mrmd_lj* lj, mrmd_atoms* a, const mrmd_nlist* nl,
                   const mrmd_pred* pred, double* ev);
}  // namespace mrmd_impl
