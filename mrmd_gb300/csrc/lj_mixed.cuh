// Split coordinates and the double-float LJ pair evaluation of the mixed form.
#pragma once

#include "lj_impl.cuh"

namespace mrmd_impl
{
struct SplitParams
{
    double3 origin;
    double scale;     // 2^q
    double invScale;  // 2^-q
};

// origin = grid corner; extent bounds |x - origin| for every coordinate.
SplitParams split_params(const double* origin, double extent);

__device__ __forceinline__ void split_one(double c, const SplitParams& sp, float& h, float& l)
{
    const double hd = rint(c * sp.scale) * sp.invScale;  // exact multiple of 2^-q
    h = (float)hd;                                        // exact: < 2^24 steps
    l = (float)(c - hd);
}

int split_coords(mrmd_ctx* ctx, const double* pos4, int64_t n, const SplitParams& sp, float4* hi, float4* lo);

// Full-list mixed pair force on split coordinates; writes (or adds to) the
// FP64 force of rows [0, nl->rows), energy/virial added to ev[0..1].
int lj_mixed_full(mrmd_ctx* ctx, const float4* hi, const float4* lo, double* force4, const LJDev& p, double rcSqr,
                  const mrmd_nlist* nl, double* ev, bool accumulate);

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

// One pair in the mixed form.  Returns false when outside the cutoff.
// ff: force factor (F_i = d * ff), e: pair energy, r2h: FP32 r^2, d: FP32 dx.
__device__ __forceinline__ bool pair_mixed(const float4& hi_i, const float4& lo_i, const float4& hj, const float4& lj,
                                           const LJDev& p, RcSq rc2, float& ff, float& e, float& r2h, float3& d)
{
    const df dx = fast_two_sum(hi_i.x - hj.x, lo_i.x - lj.x);
    const df dy = fast_two_sum(hi_i.y - hj.y, lo_i.y - lj.y);
    const df dz = fast_two_sum(hi_i.z - hj.z, lo_i.z - lj.z);
    const df r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
    if (r2.h > rc2.h || (r2.h == rc2.h && r2.l > rc2.l)) return false;  // distSqr > rcSqr
    r2h = r2.h;
    d = make_float3(dx.h, dy.h, dz.h);
    if (r2.h >= p.capSqrf)
    {
        const df u = df_rcp(r2);
        const df u2 = df_sqr(u);
        const df u3 = df_mul(u2, u);
        const df u4 = df_sqr(u2);
        const df t = df_add(df_mul(df{p.ff1h, p.ff1l}, u3), df{-p.ff2h, -p.ff2l});
        const df f = df_mul(u4, t);
        ff = f.h + f.l;
        e = __fmaf_rn(u3.h, __fmaf_rn(p.ef1f, u3.h, -p.ef2f), -p.shiftf);
    }
    else
    {
        // capped branch (action/LennardJones.hpp:70-77): |F| constant, no
        // amplification of the r^2 error
        const float dist = sqrtf(r2.h);
        ff = p.capCoeff_f / dist;
        e = p.eCapf - (dist - p.capDistf) * p.capCoeff_f - p.shiftf;
    }
    return true;
}
}  // namespace mrmd_impl
