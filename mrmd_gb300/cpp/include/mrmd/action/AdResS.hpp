// Drop-in AdResS actions: weighting_function::Slab (weighting_function/Slab.hpp:27-201),
// action::UpdateMolecules (action/UpdateMolecules.hpp:24-70),
// action::ContributeMoleculeForceToAtoms (action/ContributeMoleculeForceToAtoms.cpp:23-48),
// action::LJ_IdealGas (action/LJ_IdealGas.hpp:34-104) and
// action::ThermodynamicForce (action/ThermodynamicForce.hpp:32-96).
#pragma once

#include <vector>

#include "../data/Atoms.hpp"
#include "../data/Subdomain.hpp"

namespace mrmd
{
namespace weighting_function
{
class Slab
{
public:
    enum class InterfaceType
    {
        SMOOTH,
        ABRUPT
    };
    Slab(const Point3D& center, const real_t atomisticRegionDiameter, const real_t hybridRegionDiameter,
         const idx_t nu, const InterfaceType interfaceType = InterfaceType::SMOOTH)
    {
        s = mrmd_slab{{center[0], center[1], center[2]}, atomisticRegionDiameter, hybridRegionDiameter, nu,
                      interfaceType == InterfaceType::ABRUPT ? 1 : 0, 0};
    }
    mrmd_slab s{};
};
}  // namespace weighting_function

namespace action
{
namespace UpdateMolecules
{
inline void update(data::Molecules& molecules, const data::Atoms& atoms, const weighting_function::Slab& weight)
{
    impl::check(mrmd_update_molecules(impl::context(), molecules.raw(), atoms.raw(), &weight.s),
                "UpdateMolecules::update");
}
}  // namespace UpdateMolecules

namespace ContributeMoleculeForceToAtoms
{
inline void update(const data::Molecules& molecules, data::Atoms& atoms)
{
    impl::check(mrmd_contribute_molecule_force(impl::context(), molecules.raw(), atoms.raw()),
                "ContributeMoleculeForceToAtoms::update");
}
}  // namespace ContributeMoleculeForceToAtoms

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
        impl::check(mrmd_ljig_create(impl::context(), &s_, numTypes, cappingDistance.data(), rc.data(),
                                     sigma.data(), epsilon.data(), doShift ? 1 : 0),
                    "LJ_IdealGas");
    }
    ~LJ_IdealGas() { mrmd_ljig_destroy(impl::context(), s_); }
    LJ_IdealGas(const LJ_IdealGas&) = delete;
    LJ_IdealGas& operator=(const LJ_IdealGas&) = delete;

    void setCompensationEnergySamplingInterval(const idx_t& interval)
    {
        sampling_ = interval;
        impl::check(mrmd_ljig_set_intervals(s_, sampling_, update_), "interval");
    }
    void setCompensationEnergyUpdateInterval(const idx_t& interval)
    {
        update_ = interval;
        impl::check(mrmd_ljig_set_intervals(s_, sampling_, update_), "interval");
    }
    std::vector<real_t> getMeanCompensationEnergy() const
    {
        std::vector<real_t> mean(200 * numTypes_);
        impl::check(mrmd_ljig_get_compensation(impl::context(), s_, mean.data(), nullptr, nullptr, nullptr),
                    "getMeanCompensationEnergy");
        return mean;
    }

    real_t run(data::Molecules& molecules, HalfVerletList& verletList, data::Atoms& atoms)
    {
        real_t e = 0_r;
        impl::check(mrmd_ljig_run(impl::context(), s_, molecules.raw(), verletList.raw(), atoms.raw(), precision, &e),
                    "LJ_IdealGas::run");
        return e;
    }

    int precision = MRMD_PREC_FP64;

private:
    mrmd_ljig* s_ = nullptr;
    idx_t numTypes_ = 1;
    idx_t sampling_ = 200, update_ = 20000;
};

class ThermodynamicForce
{
public:
    ThermodynamicForce(const std::vector<real_t>& targetDensity, const data::Subdomain& subdomain,
                       const real_t& requestedDensityBinWidth, const std::vector<real_t>& thermodynamicForceModulation,
                       const bool enforceSymmetry = false, const bool usePeriodicity = false)
    {
        impl::check(mrmd_tf_create(impl::context(), &tf_, idx_t(targetDensity.size()), targetDensity.data(),
                                   &subdomain.s, requestedDensityBinWidth, thermodynamicForceModulation.data(),
                                   enforceSymmetry ? 1 : 0, usePeriodicity ? 1 : 0),
                    "ThermodynamicForce");
        mrmd_tf_shape(tf_, &numBins_, &binSize_, &numTypes_);
    }
    ThermodynamicForce(const real_t targetDensity, const data::Subdomain& subdomain,
                       const real_t& requestedDensityBinWidth, const real_t thermodynamicForceModulation,
                       const bool enforceSymmetry = false, const bool usePeriodicity = false)
        : ThermodynamicForce(std::vector<real_t>{targetDensity}, subdomain, requestedDensityBinWidth,
                             std::vector<real_t>{thermodynamicForceModulation}, enforceSymmetry, usePeriodicity)
    {
    }
    // Takes ownership of a table the library made (io::restoreThermoForce).
    explicit ThermodynamicForce(mrmd_tf* adopted) : tf_(adopted)
    {
        mrmd_tf_shape(tf_, &numBins_, &binSize_, &numTypes_);
    }
    ~ThermodynamicForce() { mrmd_tf_destroy(impl::context(), tf_); }
    ThermodynamicForce(const ThermodynamicForce&) = delete;
    ThermodynamicForce& operator=(const ThermodynamicForce&) = delete;

    void sample(data::Atoms& atoms) { impl::check(mrmd_tf_sample(impl::context(), tf_, atoms.raw()), "sample"); }
    void apply(data::Atoms& atoms) const
    {
        impl::check(mrmd_tf_apply(impl::context(), tf_, atoms.raw(), nullptr, 0), "apply");
    }
    void apply_if(data::Atoms& atoms, const mrmd_pred& pred) const
    {
        impl::check(mrmd_tf_apply(impl::context(), tf_, atoms.raw(), &pred, 0), "apply_if");
    }
    void applyInterpolated_if(data::Atoms& atoms, const mrmd_pred& pred) const
    {
        impl::check(mrmd_tf_apply(impl::context(), tf_, atoms.raw(), &pred, 1), "applyInterpolated_if");
    }
    void update(const real_t& smoothingSigma, const real_t& smoothingIntensity)
    {
        impl::check(mrmd_tf_update(impl::context(), tf_, smoothingSigma, smoothingIntensity, nullptr), "update");
    }
    void update_if(const real_t& smoothingSigma, const real_t& smoothingIntensity, const mrmd_pred& pred)
    {
        impl::check(mrmd_tf_update(impl::context(), tf_, smoothingSigma, smoothingIntensity, &pred), "update_if");
    }
    std::vector<real_t> getForce() const
    {
        std::vector<real_t> f(numBins_ * numTypes_);
        impl::check(mrmd_tf_get_force(impl::context(), tf_, f.data()), "getForce");
        return f;
    }
    void setForce(const std::vector<real_t>& f)
    {
        impl::check(mrmd_tf_set_force(impl::context(), tf_, f.data()), "setForce");
    }
    std::vector<real_t> getDensityProfile() const
    {
        std::vector<real_t> d(numBins_ * numTypes_);
        impl::check(mrmd_tf_get_density(impl::context(), tf_, d.data(), nullptr), "getDensityProfile");
        return d;
    }
    std::vector<real_t> getMuLeft() const { return mu().first; }
    std::vector<real_t> getMuRight() const { return mu().second; }
    idx_t numBins() const { return numBins_; }
    idx_t numTypes() const { return numTypes_; }
    // createGrid(getForce()): the bin centres.
    std::vector<real_t> getGrid() const
    {
        std::vector<real_t> g(numBins_);
        impl::check(mrmd_tf_grid(tf_, g.data()), "getGrid");
        return g;
    }
    const mrmd_tf* raw() const { return tf_; }

private:
    std::pair<std::vector<real_t>, std::vector<real_t>> mu() const
    {
        std::vector<real_t> l(numTypes_), r(numTypes_);
        impl::check(mrmd_tf_mu(impl::context(), tf_, l.data(), r.data()), "mu");
        return {l, r};
    }
    mrmd_tf* tf_ = nullptr;
    int64_t numBins_ = 0, numTypes_ = 0;
    double binSize_ = 0;
};
}  // namespace action
}  // namespace mrmd
