// Drop-in util::IsInSymmetricSlab (util/IsInSymmetricSlab.hpp:24-64) as the
// predicate forms the GPU kernels evaluate: a one-position predicate, and
// either / both combinations of two positions for LennardJones::apply_if.
#pragma once

#include "../datatypes.hpp"

namespace mrmd::util
{
class IsInSymmetricSlab
{
public:
    IsInSymmetricSlab(const Point3D& center, const real_t slabMin, const real_t slabMax, const AXIS axis = AXIS::X,
                      const real_t tolerance = 0_r)
    {
        const int ax = int(axis);
        p_ = mrmd_pred{MRMD_PRED_IN_SLAB, ax, center[ax], slabMin, slabMax, tolerance};
    }
    mrmd_pred one() const { return p_; }
    TwoPositionsPredicate either() const  // slab(x1) || slab(x2)
    {
        TwoPositionsPredicate t{p_};
        t.p.kind = MRMD_PRED_EITHER_IN_SLAB;
        return t;
    }
    TwoPositionsPredicate both() const  // slab(x1) && slab(x2)
    {
        TwoPositionsPredicate t{p_};
        t.p.kind = MRMD_PRED_BOTH_IN_SLAB;
        return t;
    }

private:
    mrmd_pred p_{};
};
}  // namespace mrmd::util
