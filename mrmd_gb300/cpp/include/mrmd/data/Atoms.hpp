// Drop-in data::Atoms / data::HostAtoms (data/Atoms.hpp:33-177).
//
// Atoms owns device storage through the C ABI (pos/vel/force packed four
// doubles per atom).  HostAtoms is a plain host mirror in the reference's
// AoS layout; deep_copy moves data between the two as data::deep_copy does.
#pragma once

#include <vector>

#include "../datatypes.hpp"

namespace mrmd::data
{
struct HostAtoms
{
    explicit HostAtoms(idx_t n = 0) { resize(n); }
    void resize(idx_t n)
    {
        pos.resize(3 * n);
        vel.resize(3 * n);
        force.resize(3 * n);
        type.resize(n);
        mass.resize(n);
        charge.resize(n);
        relativeMass.resize(n);
    }
    idx_t size() const { return idx_t(mass.size()); }
    std::vector<real_t> pos, vel, force;
    std::vector<idx_t> type;
    std::vector<real_t> mass, charge, relativeMass;
    idx_t numLocalAtoms = 0;
    idx_t numGhostAtoms = 0;
};

class Atoms
{
public:
    explicit Atoms(idx_t numAtoms) { gb300::check(mrmd_atoms_alloc(gb300::context(), &a_, numAtoms), "Atoms"); }
    ~Atoms() { mrmd_atoms_free(gb300::context(), &a_); }
    Atoms(const Atoms&) = delete;
    Atoms& operator=(const Atoms&) = delete;

    // device arrays (pos/vel/force: [capacity][4] doubles)
    double* getPos() const { return a_.pos; }
    double* getVel() const { return a_.vel; }
    double* getForce() const { return a_.force; }
    void setForce(const real_t& val) { gb300::check(mrmd_atoms_set_force(gb300::context(), &a_, size(), val), "setForce"); }
    idx_t size() const { return a_.numLocal + a_.numGhost; }
    void resize(idx_t n) { gb300::check(mrmd_atoms_reserve(gb300::context(), &a_, n), "resize"); }

    mrmd_atoms* raw() { return &a_; }
    const mrmd_atoms* raw() const { return &a_; }

    // numLocalAtoms / numGhostAtoms (data/Atoms.hpp:120-121) live in the ABI struct
    idx_t& numLocalAtoms = a_.numLocal;
    idx_t& numGhostAtoms = a_.numGhost;

private:
    mrmd_atoms a_{};
};

// data::deep_copy(dst, src) between host and device (data/Atoms.hpp:150-159)
inline void deep_copy(Atoms& dst, const HostAtoms& src)
{
    gb300::check(mrmd_atoms_upload(gb300::context(), dst.raw(), src.numLocalAtoms, src.numGhostAtoms, src.pos.data(),
                                  src.vel.data(), src.force.data(), src.type.data(), src.mass.data(),
                                  src.charge.data(), src.relativeMass.data()),
                "deep_copy");
}

inline void deep_copy(HostAtoms& dst, const Atoms& src)
{
    dst.resize(src.size());
    dst.numLocalAtoms = src.raw()->numLocal;
    dst.numGhostAtoms = src.raw()->numGhost;
    gb300::check(mrmd_atoms_download(gb300::context(), src.raw(), src.size(), dst.pos.data(), dst.vel.data(),
                                    dst.force.data(), dst.type.data(), dst.mass.data(), dst.charge.data(),
                                    dst.relativeMass.data()),
                "deep_copy");
}
}  // namespace mrmd::data

// data::Molecules is declared in its own header, as in the reference; it is
// included here too for drivers that reach it through this one.
#include "Molecules.hpp"
