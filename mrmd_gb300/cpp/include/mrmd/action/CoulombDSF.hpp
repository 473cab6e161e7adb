// Drop-in action::impl::CoulombDSF (action/CoulombDSF.hpp:39-83): the damped
// shifted-force Coulomb pair function with the reference's approximate erfc.
// computeForce / computeEnergy evaluate single pairs on the device (the
// reference's are device functions); evaluate() takes many pairs per call.
// apply() is the pair force over a half list with the atoms' charges, in the
// loop of LennardJones::apply; the reference ships the pair function only.
#pragma once

#include <vector>

#include "../data/Atoms.hpp"

namespace mrmd::action
{
namespace impl
{
class CoulombDSF
{
public:
    CoulombDSF(const real_t& rc, const real_t& alpha)
    {
        gb300::check(mrmd_coulomb_dsf_init(&p_, rc, alpha), "CoulombDSF");
    }

    // force / distSqr of one pair (CoulombDSF.hpp:52-61)
    real_t computeForce(const real_t& distSqr, const real_t q1, const real_t q2) const
    {
        real_t f = 0_r, e = 0_r;
        evaluate(1, &distSqr, &q1, &q2, &f, &e);
        return f;
    }
    // energy of one pair (CoulombDSF.hpp:67-74)
    real_t computeEnergy(const real_t& distSqr, const real_t q1, const real_t q2) const
    {
        real_t f = 0_r, e = 0_r;
        evaluate(1, &distSqr, &q1, &q2, &f, &e);
        return e;
    }
    // n pairs from host arrays
    void evaluate(const idx_t n, const real_t* distSqr, const real_t* q1, const real_t* q2, real_t* force,
                  real_t* energy) const
    {
        gb300::check(
            mrmd_coulomb_dsf_eval(gb300::context(), &p_, n, distSqr, q1, q2, force, energy), "CoulombDSF");
    }

    // forces on i and j (ghosts included; the caller folds ghost forces back)
    void apply(data::Atoms& atoms, const HalfVerletList& verletList)
    {
        gb300::check(mrmd_coulomb_dsf_apply(gb300::context(), &p_, atoms.raw(), verletList.raw(),
                                                 &energy_, &virial_),
                          "CoulombDSF::apply");
    }
    real_t getEnergy() const { return energy_; }
    real_t getVirial() const { return virial_; }

private:
    mrmd_coulomb_dsf_params p_{};
    real_t energy_ = 0_r;
    real_t virial_ = 0_r;
};
}  // namespace impl
}  // namespace mrmd::action
