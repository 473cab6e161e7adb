// Split coordinates and the double-float LJ pair evaluation of the mixed form.
#pragma once

#include "f32_round.cuh"
#include "lj_impl.cuh"

namespace mrmd_impl
{
struct SplitParams
{
    double3 origin;
    double scale;     // 2^q
    double invScale;  // 2^-q
    double magic;     // 1.5 * 2^(52 - q)
    float invScaleF;  // 2^-q
    longlong3 ko;     // origin / 2^-q (the tile split, split_bits; origin a multiple of 2^-q)
    int q;
};

// origin = grid corner; extent bounds |x - origin| for every coordinate.
SplitParams split_params(const double* origin, double extent);

// hi = c rounded to the nearest multiple of 2^-q (ties to even) and
// lo = c - hi rounded to FP32.  The rounding is the magic-number addition
// t = c + 1.5 * 2^(52 - q): t has ulp 2^-q, so t - magic is hi exactly and the
// low word of t's bits is the integer k = hi * 2^q (|k| < 2^24), converted
// to FP32 without the FP64 pipe; four FP64 operations per coordinate.
__device__ __forceinline__ void split_one(double c, const SplitParams& sp, float& h, float& l)
{
    const double t = __dadd_rn(c, sp.magic);
    const int k = __double2loint(t);
    h = __int2float_rn(k) * sp.invScaleF;  // exact: |k| < 2^24, power-of-two scale
    l = __double2float_rn(__dsub_rn(c, __dsub_rn(t, sp.magic)));
}

// The split parameters for quantum 2^-q given by `invScale`.
__host__ __device__ inline SplitParams make_split(double scale, double invScale)
{
    SplitParams s{};
    s.scale = scale;
    s.invScale = invScale;
    s.magic = 6755399441055744.0 * invScale;  // 1.5 * 2^52 * 2^-q
    s.invScaleF = (float)invScale;
    return s;
}

// hi[i * stride], lo[i * stride] (stride 2 with lo = hi + 1: one 32-byte
// record per particle).
int split_coords(mrmd_ctx* ctx, const double* pos4, int64_t n, const SplitParams& sp, float4* hi, float4* lo,
                 int stride = 1);

// The r_split of the mixed pair kernels for LJ parameters sigma and capping distance:
// 1.4 sigma, and beyond the capping distance (the FP32 path has no cap).
inline double lj_split_radius(double sigma, double cappingDistance)
{
    const double r = 1.4 * sigma;
    return r > 1.05 * cappingDistance ? r : 1.05 * cappingDistance;
}

// Half-list mixed pair force on given split coordinates (i and j forces
// accumulated into the FP64 force array with atomics).
int lj_mixed_half(mrmd_ctx* ctx, const float4* hi, const float4* lo, const mrmd_lj* lj, mrmd_atoms* a,
                  const mrmd_nlist* nl, const mrmd_pred* pred, double* ev);

// Split parameters matching the cell grid the list was built on.
SplitParams split_params_for(const mrmd_nlist* nl);

// rc^2 as a double-float, so that the cutoff test decides on the full
// ~2^-48 accurate r^2: the LJ force jumps at rc (the shifted potential is
// continuous, its force is not), and an FP32-rounded test would misplace
// the pairs within 2^-24 of rc^2.
struct RcSq
{
    float h, l;
};

inline RcSq make_rcsq(double rcSqr)
{
    RcSq r;
    r.h = (float)rcSqr;
    r.l = (float)(rcSqr - (double)r.h);
    return r;
}

// Result of one pair in the mixed form.  dx = dh + dl exactly (the split
// coordinates make hi_i - hi_j exact), ff is the double-float force factor
// (F_i += dx * ff), e the FP32 pair energy, (r2h, r2l) r^2 as a double-float.
struct PairMixed
{
    float3 dh, dl;
    df ff;
    float e, r2h, r2l;
};

// One pair in the mixed form; false when outside the cutoff (distSqr > rcSqr).
__device__ __forceinline__ bool pair_mixed(const float4& hi_i, const float4& lo_i, const float4& hj, const float4& lj,
                                           const LJDev& p, RcSq rc2, PairMixed& o)
{
    o.dh = make_float3(hi_i.x - hj.x, hi_i.y - hj.y, hi_i.z - hj.z);  // exact
    o.dl = make_float3(lo_i.x - lj.x, lo_i.y - lj.y, lo_i.z - lj.z);  // |dl| <= 2^-q
    // FP32 early reject, far outside the FP32 error of r^2
    const float fx = o.dh.x + o.dl.x, fy = o.dh.y + o.dl.y, fz = o.dh.z + o.dl.z;
    const float r2f = __fmaf_rn(fx, fx, __fmaf_rn(fy, fy, fz * fz));
    if (r2f > rc2.h * 1.0000005f) return false;
    // r^2 = sum (dh + dl)^2 as double-float: exact squares of the heads
    // (FMA TwoProd), the 2*dh*dl cross terms and dl^2 in the low part (dl^2
    // matters for close contacts, where |dl| is not small against |dh|)
    const float px = o.dh.x * o.dh.x, py = o.dh.y * o.dh.y, pz = o.dh.z * o.dh.z;
    float lo = __fmaf_rn(o.dl.x, o.dl.x, __fmaf_rn(o.dl.y, o.dl.y, o.dl.z * o.dl.z));
    lo += __fmaf_rn(o.dh.x, o.dh.x, -px);
    lo += __fmaf_rn(o.dh.y, o.dh.y, -py);
    lo += __fmaf_rn(o.dh.z, o.dh.z, -pz);
    lo = __fmaf_rn(2.0f * o.dh.x, o.dl.x, lo);
    lo = __fmaf_rn(2.0f * o.dh.y, o.dl.y, lo);
    lo = __fmaf_rn(2.0f * o.dh.z, o.dl.z, lo);
    const df s1 = two_sum(px, py);
    const df s2 = two_sum(s1.h, pz);
    const df r2 = fast_two_sum(s2.h, s2.l + s1.l + lo);
    if (r2.h > rc2.h || (r2.h == rc2.h && r2.l > rc2.l)) return false;
    o.r2h = r2.h;
    o.r2l = r2.l;
    if (r2.h >= p.capSqrf)
    {
        const df u = df_rcp(r2);
        const df u2 = df_sqr(u);
        const df u3 = df_mul(u2, u);
        const df u4 = df_sqr(u2);
        const df t = df_add(df_mul(df{p.ff1h, p.ff1l}, u3), df{-p.ff2h, -p.ff2l});
        o.ff = df_mul(u4, t);
        o.e = __fmaf_rn(u3.h, __fmaf_rn(p.ef1f, u3.h, -p.ef2f), -p.shiftf);
    }
    else
    {
        // capped branch (action/LennardJones.hpp:70-77): |F| = capCoeff is
        // constant, so forceFactor = capCoeff / r carries the relative error
        // of r straight into the force: r and 1/r as double-floats
        const df dist = df_sqrt(r2);
        o.ff = df_mul(df{p.capCoeff_f, p.capCoeff_l}, df_rcp(dist));
        o.e = p.eCapf - (dist.h - p.capDistf) * p.capCoeff_f - p.shiftf;
    }
    return true;
}

// s += (dh + dl) * ff in double-float (FMA TwoProd of the heads, first-order
// cross terms), so no pair force is ever rounded to FP32.
__device__ __forceinline__ void df_acc_prod(df& s, float dh, float dl, const df& ff)
{
    const float p = dh * ff.h;
    float e = __fmaf_rn(dh, ff.h, -p);
    e = __fmaf_rn(dh, ff.l, e);
    e = __fmaf_rn(dl, ff.h, e);
    const df t = two_sum(s.h, p);
    s.h = t.h;
    s.l += t.l + e;
}

// The same product as a double (for FP64 atomics of the j-force).
__device__ __forceinline__ double prod_d(float dh, float dl, const df& ff)
{
    const float p = dh * ff.h;
    float e = __fmaf_rn(dh, ff.h, -p);
    e = __fmaf_rn(dh, ff.l, e);
    e = __fmaf_rn(dl, ff.h, e);
    return (double)p + (double)e;
}
}  // namespace mrmd_impl
