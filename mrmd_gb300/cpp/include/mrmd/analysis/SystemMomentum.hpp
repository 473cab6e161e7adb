// Drop-in analysis::getSystemMomentum (analysis/SystemMomentum.cpp:21-48):
// the sum of the local atoms' velocities (the reference applies no mass
// factor), summed on the device in a fixed order.
#pragma once

#include "../data/Atoms.hpp"

namespace mrmd::analysis
{
inline Vector3D getSystemMomentum(data::Atoms& atoms)
{
    Vector3D p{0_r, 0_r, 0_r};
    gb300::check(mrmd_system_momentum(gb300::context(), atoms.raw(), p.data()), "getSystemMomentum");
    return p;
}
}  // namespace mrmd::analysis
