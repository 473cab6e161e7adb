// Drop-in action::UpdateMolecules (action/UpdateMolecules.hpp:24-70).
#pragma once

#include "../data/Atoms.hpp"
#include "../data/Molecules.hpp"
#include "../weighting_function/Slab.hpp"

namespace mrmd::action
{
namespace UpdateMolecules
{
inline void update(data::Molecules& molecules, const data::Atoms& atoms, const weighting_function::Slab& weight)
{
    gb300::check(mrmd_update_molecules(gb300::context(), molecules.raw(), atoms.raw(), &weight.s),
                "UpdateMolecules::update");
}
}  // namespace UpdateMolecules
}  // namespace mrmd::action
