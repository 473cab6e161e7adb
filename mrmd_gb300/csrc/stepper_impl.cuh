// Asynchronous building blocks of the fused steppers (no host read-back).
#pragma once

#include "common.cuh"

namespace mrmd_impl
{
// VelocityVerletLangevinThermostat::preForceIntegrate; max |dx|^2 via atomicMax into dMax.
int langevin_pre_async(mrmd_ctx* ctx, mrmd_atoms* a, double dt, double zeta, double temperature, uint64_t seed,
                       uint64_t step, const mrmd_pred* pred, double* dMax);
// LJ_IdealGas::run, energy added to *ev (device); hi/lo: precomputed split
// coordinates for the mixed form or null.
int ljig_run_async(mrmd_ctx* ctx, mrmd_ljig* s, mrmd_molecules* m, const mrmd_nlist* nl, mrmd_atoms* a,
                   int precision, double* ev, const float4* hi, const float4* lo);
}  // namespace mrmd_impl
