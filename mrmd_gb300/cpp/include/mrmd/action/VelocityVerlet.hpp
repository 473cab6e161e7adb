// Drop-in action::VelocityVerlet (action/VelocityVerlet.hpp:26-31).
#pragma once

#include "../data/Atoms.hpp"

namespace mrmd::action
{
class VelocityVerlet
{
public:
    static real_t preForceIntegrate(data::Atoms& atoms, const real_t dt)
    {
        real_t maxDisp = 0_r;
        gb300::check(mrmd_vv_pre(gb300::context(), atoms.raw(), dt, &maxDisp), "preForceIntegrate");
        return maxDisp;
    }
    static void postForceIntegrate(data::Atoms& atoms, const real_t dt)
    {
        gb300::check(mrmd_vv_post(gb300::context(), atoms.raw(), dt), "postForceIntegrate");
    }
};
}  // namespace mrmd::action
