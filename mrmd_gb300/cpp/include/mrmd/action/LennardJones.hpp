// Drop-in action::LennardJones (action/LennardJones.hpp:98-133).
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
    // the reference indexes its table with numTypes_ fixed to 1 (action/LennardJones.cpp:52)
    LennardJones(const std::vector<real_t>& cappingDistance, const std::vector<real_t>& rc,
                 const std::vector<real_t>& sigma, const std::vector<real_t>& epsilon, const idx_t& numTypes,
                 const bool isShifted)
    {
        gb300::check(mrmd_lj_create(gb300::context(), &lj_, numTypes, 1, cappingDistance.data(), rc.data(),
                                   sigma.data(), epsilon.data(), isShifted ? 1 : 0),
                    "LennardJones");
    }
    ~LennardJones() { mrmd_lj_destroy(gb300::context(), lj_); }
    LennardJones(const LennardJones&) = delete;
    LennardJones& operator=(const LennardJones&) = delete;

    void apply(data::Atoms& atoms, HalfVerletList& verletList) { apply_if(atoms, verletList, TwoPositionsPredicate{}); }

    void apply_if(const data::Atoms& atoms, const HalfVerletList& verletList, const TwoPositionsPredicate& pred)
    {
        gb300::check(mrmd_lj_apply(gb300::context(), lj_, const_cast<mrmd_atoms*>(atoms.raw()), verletList.raw(),
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
}  // namespace mrmd::action

// The integrators have their own headers, as in the reference; they are
// included here too for drivers that reach them through this one.
#include "VelocityVerlet.hpp"
#include "VelocityVerletLangevinThermostat.hpp"
