// Drop-in action::LJ_IdealGas (action/LJ_IdealGas.hpp:34-104).
#pragma once

#include <vector>

#include "../data/Atoms.hpp"
#include "../data/Molecules.hpp"

namespace mrmd::action
{
class LJ_IdealGas
{
public:
    LJ_IdealGas(const real_t& cappingDistance, const real_t& rc, const real_t& sigma, const real_t& epsilon,
                const bool doShift)
        : LJ_IdealGas(std::vector<real_t>{cappingDistance}, {rc}, {sigma}, {epsilon}, 1, doShift)
    {
    }
    LJ_IdealGas(const std::vector<real_t>& cappingDistance, const std::vector<real_t>& rc,
                const std::vector<real_t>& sigma, const std::vector<real_t>& epsilon, const idx_t numTypes,
                const bool doShift)
        : numTypes_(numTypes)
    {
        gb300::check(mrmd_ljig_create(gb300::context(), &s_, numTypes, cappingDistance.data(), rc.data(),
                                     sigma.data(), epsilon.data(), doShift ? 1 : 0),
                    "LJ_IdealGas");
    }
    ~LJ_IdealGas() { mrmd_ljig_destroy(gb300::context(), s_); }
    LJ_IdealGas(const LJ_IdealGas&) = delete;
    LJ_IdealGas& operator=(const LJ_IdealGas&) = delete;

    void setCompensationEnergySamplingInterval(const idx_t& interval)
    {
        sampling_ = interval;
        gb300::check(mrmd_ljig_set_intervals(s_, sampling_, update_), "interval");
    }
    void setCompensationEnergyUpdateInterval(const idx_t& interval)
    {
        update_ = interval;
        gb300::check(mrmd_ljig_set_intervals(s_, sampling_, update_), "interval");
    }
    std::vector<real_t> getMeanCompensationEnergy() const
    {
        std::vector<real_t> mean(200 * numTypes_);
        gb300::check(mrmd_ljig_get_compensation(gb300::context(), s_, mean.data(), nullptr, nullptr, nullptr),
                    "getMeanCompensationEnergy");
        return mean;
    }

    real_t run(data::Molecules& molecules, HalfVerletList& verletList, data::Atoms& atoms)
    {
        real_t e = 0_r;
        gb300::check(mrmd_ljig_run(gb300::context(), s_, molecules.raw(), verletList.raw(), atoms.raw(), precision, &e),
                    "LJ_IdealGas::run");
        return e;
    }

    int precision = MRMD_PREC_FP64;

private:
    mrmd_ljig* s_ = nullptr;
    idx_t numTypes_ = 1;
    idx_t sampling_ = 200, update_ = 20000;
};
}  // namespace mrmd::action
