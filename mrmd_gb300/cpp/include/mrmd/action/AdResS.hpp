// The AdResS actions of the drop-in in one include: weighting_function::Slab,
// action::UpdateMolecules, action::ContributeMoleculeForceToAtoms,
// action::LJ_IdealGas and action::ThermodynamicForce, each in the header of
// the reference's path.
#pragma once

#include "../weighting_function/Slab.hpp"
#include "ContributeMoleculeForceToAtoms.hpp"
#include "LJ_IdealGas.hpp"
#include "ThermodynamicForce.hpp"
#include "UpdateMolecules.hpp"
