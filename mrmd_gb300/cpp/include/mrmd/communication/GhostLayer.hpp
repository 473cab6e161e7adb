// Drop-in communication::GhostLayer (communication/GhostLayer.hpp:28-56) and
// communication::MultiResGhostLayer (communication/MultiResGhostLayer.hpp:29-61).
#pragma once

#include "../data/Atoms.hpp"
#include "../data/Subdomain.hpp"

namespace mrmd::communication
{
class GhostLayer
{
public:
    GhostLayer() { impl::check(mrmd_ghost_layer_alloc(impl::context(), &g_, 1), "GhostLayer"); }
    ~GhostLayer() { mrmd_ghost_layer_free(impl::context(), &g_); }
    GhostLayer(const GhostLayer&) = delete;
    GhostLayer& operator=(const GhostLayer&) = delete;

    void exchangeRealAtoms(data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        impl::check(mrmd_ghost_exchange_real_atoms(impl::context(), atoms.raw(), &subdomain.s), "exchangeRealAtoms");
    }
    void createGhostAtoms(data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        impl::check(mrmd_ghost_create(impl::context(), &g_, atoms.raw(), &subdomain.s), "createGhostAtoms");
    }
    void updateGhostAtoms(data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        impl::check(mrmd_ghost_update(impl::context(), &g_, atoms.raw(), &subdomain.s), "updateGhostAtoms");
    }
    void contributeBackGhostToReal(data::Atoms& atoms)
    {
        impl::check(mrmd_ghost_reduce_force(impl::context(), &g_, atoms.raw()), "contributeBackGhostToReal");
    }

protected:
    mrmd_ghost_layer g_{};
};

class MultiResGhostLayer : public GhostLayer
{
public:
    void exchangeRealAtoms(data::Molecules& molecules, data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        impl::check(mrmd_multires_exchange_real_atoms(impl::context(), molecules.raw(), atoms.raw(), &subdomain.s),
                    "exchangeRealAtoms");
    }
    void createGhostAtoms(data::Molecules& molecules, data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        impl::check(mrmd_multires_ghost_create(impl::context(), &g_, molecules.raw(), atoms.raw(), &subdomain.s),
                    "createGhostAtoms");
    }
};
}  // namespace mrmd::communication
