// Drop-in weighting_function::Slab (weighting_function/Slab.hpp:27-201): the
// slab geometry handed to the device kernels that evaluate the weights.
#pragma once

#include "../datatypes.hpp"

namespace mrmd::weighting_function
{
class Slab
{
public:
    enum class InterfaceType
    {
        SMOOTH,
        ABRUPT
    };
    Slab(const Point3D& center, const real_t atomisticRegionDiameter, const real_t hybridRegionDiameter,
         const idx_t nu, const InterfaceType interfaceType = InterfaceType::SMOOTH)
    {
        s = mrmd_slab{{center[0], center[1], center[2]}, atomisticRegionDiameter, hybridRegionDiameter, nu,
                      interfaceType == InterfaceType::ABRUPT ? 1 : 0, 0};
    }
    mrmd_slab s{};
};
}  // namespace mrmd::weighting_function
