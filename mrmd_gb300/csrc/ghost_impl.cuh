// The periodic ghost position update of one ghost, shared by the ghost layer
// and the fused stepper.
#pragma once

#include "common.cuh"

namespace mrmd_impl
{
// communication/UpdateGhostAtoms.cpp:31-68: the ghost takes its real atom's
// position shifted by the box length along every axis where its old position
// was more than delta away from the real atom.
__device__ __forceinline__ double4 ghost_position(const double4& old, const double4& r, const double3& L,
                                                  const double3& delta)
{
    const double dx = __dsub_rn(old.x, r.x), dy = __dsub_rn(old.y, r.y), dz = __dsub_rn(old.z, r.z);
    double4 p = r;
    if (dx > +delta.x) p.x = __dadd_rn(p.x, L.x);
    if (dy > +delta.y) p.y = __dadd_rn(p.y, L.y);
    if (dz > +delta.z) p.z = __dadd_rn(p.z, L.z);
    if (dx < -delta.x) p.x = __dsub_rn(p.x, L.x);
    if (dy < -delta.y) p.y = __dsub_rn(p.y, L.y);
    if (dz < -delta.z) p.z = __dsub_rn(p.z, L.z);
    p.w = 0.0;
    return p;
}
}  // namespace mrmd_impl
