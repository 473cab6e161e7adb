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
    GhostLayer() { gb300::check(mrmd_ghost_layer_alloc(gb300::context(), &g_, 1), "GhostLayer"); }
    ~GhostLayer() { mrmd_ghost_layer_free(gb300::context(), &g_); }
    GhostLayer(const GhostLayer&) = delete;
    GhostLayer& operator=(const GhostLayer&) = delete;

    void exchangeRealAtoms(data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        gb300::check(mrmd_ghost_exchange_real_atoms(gb300::context(), atoms.raw(), &subdomain.s), "exchangeRealAtoms");
    }
    void createGhostAtoms(data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        gb300::check(mrmd_ghost_create(gb300::context(), &g_, atoms.raw(), &subdomain.s), "createGhostAtoms");
    }
    void updateGhostAtoms(data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        gb300::check(mrmd_ghost_update(gb300::context(), &g_, atoms.raw(), &subdomain.s), "updateGhostAtoms");
    }
    void contributeBackGhostToReal(data::Atoms& atoms)
    {
        gb300::check(mrmd_ghost_reduce_force(gb300::context(), &g_, atoms.raw()), "contributeBackGhostToReal");
    }

protected:
    mrmd_ghost_layer g_{};
};

class MultiResGhostLayer : public GhostLayer
{
public:
    void exchangeRealAtoms(data::Molecules& molecules, data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        gb300::check(mrmd_multires_exchange_real_atoms(gb300::context(), molecules.raw(), atoms.raw(), &subdomain.s),
                    "exchangeRealAtoms");
    }
    void createGhostAtoms(data::Molecules& molecules, data::Atoms& atoms, const data::Subdomain& subdomain)
    {
        gb300::check(mrmd_multires_ghost_create(gb300::context(), &g_, molecules.raw(), atoms.raw(), &subdomain.s),
                    "createGhostAtoms");
    }
};
}  // namespace mrmd::communication
