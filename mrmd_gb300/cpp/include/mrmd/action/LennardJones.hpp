// Drop-in action::LennardJones (action/LennardJones.hpp:98-133) and
// action::VelocityVerlet (action/VelocityVerlet.hpp:26-31).
#pragma once

#include <vector>

#include "../data/Atoms.hpp"
#include "../util/IsInSymmetricSlab.hpp"

namespace mrmd::action
{
class LennardJones
{
public:
    // LennardJones(rc, sigma, epsilon, cappingDistance): unshifted, one type
    // (LennardJones.cpp:38-44)
    LennardJones(const real_t rc, const real_t& sigma, const real_t& epsilon, const real_t& cappingDistance = 0_r)
        : LennardJones({cappingDistance}, {rc}, {sigma}, {epsilon}, 1, false)
    {
    }
    // LennardJones(cappingDistance[], rc[], sigma[], epsilon[], numTypes, isShifted);
    // the reference indexes its table with numTypes_ fixed to 1 (LennardJones.cpp:260)
    LennardJones(const std::vector<real_t>& cappingDistance, const std::vector<real_t>& rc,
                 const std::vector<real_t>& sigma, const std::vector<real_t>& epsilon, const idx_t& numTypes,
                 const bool isShifted)
    {
        impl::check(mrmd_lj_create(impl::context(), &lj_, numTypes, 1, cappingDistance.data(), rc.data(),
                                   sigma.data(), epsilon.data(), isShifted ? 1 : 0),
                    "LennardJones");
    }
    ~LennardJones() { mrmd_lj_destroy(impl::context(), lj_); }
    LennardJones(const LennardJones&) = delete;
    LennardJones& operator=(const LennardJones&) = delete;

    void apply(data::Atoms& atoms, HalfVerletList& verletList) { apply_if(atoms, verletList, TwoPositionsPredicate{}); }

    void apply_if(const data::Atoms& atoms, const HalfVerletList& verletList, const TwoPositionsPredicate& pred)
    {
        impl::check(mrmd_lj_apply(impl::context(), lj_, const_cast<mrmd_atoms*>(atoms.raw()), verletList.raw(),
                                  &pred.p, precision, &energy_, &virial_),
                    "LennardJones::apply_if");
    }

    real_t getEnergy() const { return energy_; }
    real_t getVirial() const { return virial_; }

    int precision = MRMD_PREC_FP64;  // MRMD_PREC_MIXED selects the mixed form

private:
    mrmd_lj* lj_ = nullptr;
    real_t energy_ = 0_r;
    real_t virial_ = 0_r;
};

class VelocityVerlet
{
public:
    static real_t preForceIntegrate(data::Atoms& atoms, const real_t dt)
    {
        real_t maxDisp = 0_r;
        impl::check(mrmd_vv_pre(impl::context(), atoms.raw(), dt, &maxDisp), "preForceIntegrate");
        return maxDisp;
    }
    static void postForceIntegrate(data::Atoms& atoms, const real_t dt)
    {
        impl::check(mrmd_vv_post(impl::context(), atoms.raw(), dt), "postForceIntegrate");
    }
};

// VelocityVerletLangevinThermostat (action/VelocityVerletLangevinThermostat.hpp:29-121)
// with reproducible Philox noise keyed by (seed, step).
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
        impl::check(mrmd_langevin_pre(impl::context(), atoms.raw(), dt, zeta_, temperature_, seed, step_++, &pred,
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
