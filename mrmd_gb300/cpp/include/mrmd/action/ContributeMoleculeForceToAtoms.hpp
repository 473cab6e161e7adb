// Drop-in action::ContributeMoleculeForceToAtoms
// (action/ContributeMoleculeForceToAtoms.cpp:23-48).
#pragma once

#include "../data/Atoms.hpp"
#include "../data/Molecules.hpp"

namespace mrmd::action
{
namespace ContributeMoleculeForceToAtoms
{
inline void update(const data::Molecules& molecules, data::Atoms& atoms)
{
    gb300::check(mrmd_contribute_molecule_force(gb300::context(), molecules.raw(), atoms.raw()),
                "ContributeMoleculeForceToAtoms::update");
}
}  // namespace ContributeMoleculeForceToAtoms
}  // namespace mrmd::action
