// Drop-in action::ThermodynamicForce (action/ThermodynamicForce.hpp:32-96).
#pragma once

#include <utility>
#include <vector>

#include "../data/Atoms.hpp"
#include "../data/Subdomain.hpp"

namespace mrmd::action
{
class ThermodynamicForce
{
public:
    ThermodynamicForce(const std::vector<real_t>& targetDensity, const data::Subdomain& subdomain,
                       const real_t& requestedDensityBinWidth, const std::vector<real_t>& thermodynamicForceModulation,
                       const bool enforceSymmetry = false, const bool usePeriodicity = false)
    {
        gb300::check(mrmd_tf_create(gb300::context(), &tf_, idx_t(targetDensity.size()), targetDensity.data(),
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
    ~ThermodynamicForce() { mrmd_tf_destroy(gb300::context(), tf_); }
    ThermodynamicForce(const ThermodynamicForce&) = delete;
    ThermodynamicForce& operator=(const ThermodynamicForce&) = delete;

    void sample(data::Atoms& atoms) { gb300::check(mrmd_tf_sample(gb300::context(), tf_, atoms.raw()), "sample"); }
    void apply(data::Atoms& atoms) const
    {
        gb300::check(mrmd_tf_apply(gb300::context(), tf_, atoms.raw(), nullptr, 0), "apply");
    }
    void apply_if(data::Atoms& atoms, const mrmd_pred& pred) const
    {
        gb300::check(mrmd_tf_apply(gb300::context(), tf_, atoms.raw(), &pred, 0), "apply_if");
    }
    void applyInterpolated_if(data::Atoms& atoms, const mrmd_pred& pred) const
    {
        gb300::check(mrmd_tf_apply(gb300::context(), tf_, atoms.raw(), &pred, 1), "applyInterpolated_if");
    }
    void update(const real_t& smoothingSigma, const real_t& smoothingIntensity)
    {
        gb300::check(mrmd_tf_update(gb300::context(), tf_, smoothingSigma, smoothingIntensity, nullptr), "update");
    }
    void update_if(const real_t& smoothingSigma, const real_t& smoothingIntensity, const mrmd_pred& pred)
    {
        gb300::check(mrmd_tf_update(gb300::context(), tf_, smoothingSigma, smoothingIntensity, &pred), "update_if");
    }
    std::vector<real_t> getForce() const
    {
        std::vector<real_t> f(numBins_ * numTypes_);
        gb300::check(mrmd_tf_get_force(gb300::context(), tf_, f.data()), "getForce");
        return f;
    }
    void setForce(const std::vector<real_t>& f)
    {
        gb300::check(mrmd_tf_set_force(gb300::context(), tf_, f.data()), "setForce");
    }
    std::vector<real_t> getDensityProfile() const
    {
        std::vector<real_t> d(numBins_ * numTypes_);
        gb300::check(mrmd_tf_get_density(gb300::context(), tf_, d.data(), nullptr), "getDensityProfile");
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
        gb300::check(mrmd_tf_grid(tf_, g.data()), "getGrid");
        return g;
    }
    const mrmd_tf* raw() const { return tf_; }

private:
    std::pair<std::vector<real_t>, std::vector<real_t>> mu() const
    {
        std::vector<real_t> l(numTypes_), r(numTypes_);
        gb300::check(mrmd_tf_mu(gb300::context(), tf_, l.data(), r.data()), "mu");
        return {l, r};
    }
    mrmd_tf* tf_ = nullptr;
    int64_t numBins_ = 0, numTypes_ = 0;
    double binSize_ = 0;
};
}  // namespace mrmd::action
