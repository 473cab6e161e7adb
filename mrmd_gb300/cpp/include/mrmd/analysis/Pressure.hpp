// Drop-in analysis::getPressure (analysis/Pressure.cpp:23-51): the sum over
// local and ghost atoms of m v.v + F.x over 3 * Subdomain::getVolume, summed on
// the device in a fixed order.
#pragma once

#include "../data/Atoms.hpp"
#include "../data/Subdomain.hpp"

namespace mrmd::analysis
{
inline real_t getPressure(data::Atoms& atoms, const data::Subdomain& subdomain)
{
    real_t p = 0_r;
    gb300::check(mrmd_pressure(gb300::context(), atoms.raw(), &subdomain.s, &p), "getPressure");
    return p;
}
}  // namespace mrmd::analysis
