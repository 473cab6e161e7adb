// Drop-in counterpart of io/RestoreThermoForce.hpp (defaults of
// io/RestoreThermoForce.hpp:24-31, reader io/RestoreThermoForce.cpp:24-90).
#pragma once

#include <string>
#include <vector>

#include "../action/AdResS.hpp"
#include "../data/Subdomain.hpp"

namespace mrmd
{
namespace io
{
inline action::ThermodynamicForce restoreThermoForce(
    const std::string& filename,
    const data::Subdomain& subdomain,
    const std::vector<real_t>& targetDensities = {1_r},
    const std::vector<real_t>& thermodynamicForceModulations = {1_r},
    const bool enforceSymmetry = false,
    const bool usePeriodicity = false,
    const idx_t maxNumForces = 10)
{
    if (targetDensities.size() != thermodynamicForceModulations.size())
        throw Error(MRMD_ERR_ARG, "restoreThermoForce: one modulation per target density");
    mrmd_tf* tf = nullptr;
    gb300::check(mrmd_tf_restore(gb300::context(), &tf, filename.c_str(), &subdomain.s, idx_t(targetDensities.size()),
                                targetDensities.data(), thermodynamicForceModulations.data(),
                                enforceSymmetry ? 1 : 0, usePeriodicity ? 1 : 0, maxNumForces),
                "restoreThermoForce");
    return action::ThermodynamicForce(tf);
}
}  // namespace io
}  // namespace mrmd
