// Drop-in action::VelocityVerletLangevinThermostat
// (action/VelocityVerletLangevinThermostat.hpp:29-121) with reproducible
// Philox noise keyed by (seed, step).
#pragma once

#include "../data/Atoms.hpp"
#include "VelocityVerlet.hpp"

namespace mrmd::action
{
class VelocityVerletLangevinThermostat
{
public:
    VelocityVerletLangevinThermostat(const real_t& zeta, const real_t& temperature) { set(zeta, temperature); }
    void set(const real_t& zeta, const real_t& temperature)
    {
        zeta_ = zeta;
        temperature_ = temperature;
    }
    real_t preForceIntegrate(data::Atoms& atoms, const real_t dt)
    {
        return preForceIntegrate_apply_if(atoms, dt, mrmd_pred{MRMD_PRED_ALWAYS, 0, 0, 0, 0, 0});
    }
    real_t preForceIntegrate_apply_if(data::Atoms& atoms, const real_t dt, const mrmd_pred& pred)
    {
        real_t maxDisp = 0_r;
        gb300::check(mrmd_langevin_pre(gb300::context(), atoms.raw(), dt, zeta_, temperature_, seed, step_++, &pred,
                                      &maxDisp),
                    "preForceIntegrate");
        return maxDisp;
    }
    void postForceIntegrate(data::Atoms& atoms, const real_t dt) { VelocityVerlet::postForceIntegrate(atoms, dt); }

    uint64_t seed = 1234;  // the reference seeds its pool with 1234 (:32)

private:
    real_t zeta_ = 0_r, temperature_ = 0_r;
    uint64_t step_ = 0;
};
}  // namespace mrmd::action
