// Drop-in analysis::getKineticEnergy / getMeanKineticEnergy
// (analysis/KineticEnergy.hpp:26-47), summed on the device in a fixed order.
#pragma once

#include "../data/Atoms.hpp"

namespace mrmd::analysis
{
// 0.5 sum m v.v over the local atoms
inline real_t getKineticEnergy(data::Atoms& atoms)
{
    real_t e = 0_r;
    gb300::check(mrmd_kinetic_energy(gb300::context(), atoms.raw(), &e), "getKineticEnergy");
    return e;
}

// the same per local atom
inline real_t getMeanKineticEnergy(data::Atoms& atoms)
{
    return getKineticEnergy(atoms) / static_cast<real_t>(atoms.numLocalAtoms);
}
}  // namespace mrmd::analysis
