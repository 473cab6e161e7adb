// Drop-in data::Atoms / data::HostAtoms (data/Atoms.hpp:33-177) and
// data::Molecules (data/Molecules.hpp:27-176).
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
    explicit Atoms(idx_t numAtoms) { impl::check(mrmd_atoms_alloc(impl::context(), &a_, numAtoms), "Atoms"); }
    ~Atoms() { mrmd_atoms_free(impl::context(), &a_); }
    Atoms(const Atoms&) = delete;
    Atoms& operator=(const Atoms&) = delete;

    // device arrays (pos/vel/force: [capacity][4] doubles)
    double* getPos() const { return a_.pos; }
    double* getVel() const { return a_.vel; }
    double* getForce() const { return a_.force; }
    void setForce(const real_t& val) { impl::check(mrmd_atoms_set_force(impl::context(), &a_, size(), val), "setForce"); }
    idx_t size() const { return a_.numLocal + a_.numGhost; }
    void resize(idx_t n) { impl::check(mrmd_atoms_reserve(impl::context(), &a_, n), "resize"); }

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
    impl::check(mrmd_atoms_upload(impl::context(), dst.raw(), src.numLocalAtoms, src.numGhostAtoms, src.pos.data(),
                                  src.vel.data(), src.force.data(), src.type.data(), src.mass.data(),
                                  src.charge.data(), src.relativeMass.data()),
                "deep_copy");
}

inline void deep_copy(HostAtoms& dst, const Atoms& src)
{
    dst.resize(src.size());
    dst.numLocalAtoms = src.raw()->numLocal;
    dst.numGhostAtoms = src.raw()->numGhost;
    impl::check(mrmd_atoms_download(impl::context(), src.raw(), src.size(), dst.pos.data(), dst.vel.data(),
                                    dst.force.data(), dst.type.data(), dst.mass.data(), dst.charge.data(),
                                    dst.relativeMass.data()),
                "deep_copy");
}

struct HostMolecules
{
    explicit HostMolecules(idx_t n = 0) { resize(n); }
    void resize(idx_t n)
    {
        pos.resize(3 * n);
        force.resize(3 * n);
        lambda.resize(n);
        modulatedLambda.resize(n);
        gradLambda.resize(3 * n);
        atomsOffset.resize(n);
        numAtoms.resize(n);
    }
    idx_t size() const { return idx_t(lambda.size()); }
    std::vector<real_t> pos, force, lambda, modulatedLambda, gradLambda;
    std::vector<idx_t> atomsOffset, numAtoms;
    idx_t numLocalMolecules = 0;
    idx_t numGhostMolecules = 0;
};

class Molecules
{
public:
    explicit Molecules(idx_t n) { impl::check(mrmd_molecules_alloc(impl::context(), &m_, n), "Molecules"); }
    ~Molecules() { mrmd_molecules_free(impl::context(), &m_); }
    Molecules(const Molecules&) = delete;
    Molecules& operator=(const Molecules&) = delete;

    double* getPos() const { return m_.pos; }
    void setForce(const real_t& val)
    {
        impl::check(mrmd_molecules_set_force(impl::context(), &m_, size(), val), "setForce");
    }
    idx_t size() const { return m_.numLocal + m_.numGhost; }
    mrmd_molecules* raw() { return &m_; }
    const mrmd_molecules* raw() const { return &m_; }

    idx_t& numLocalMolecules = m_.numLocal;
    idx_t& numGhostMolecules = m_.numGhost;

private:
    mrmd_molecules m_{};
};

inline void deep_copy(Molecules& dst, const HostMolecules& src)
{
    impl::check(mrmd_molecules_upload(impl::context(), dst.raw(), src.numLocalMolecules, src.numGhostMolecules,
                                      src.pos.data(), src.force.data(), src.lambda.data(),
                                      src.modulatedLambda.data(), src.gradLambda.data(), src.atomsOffset.data(),
                                      src.numAtoms.data()),
                "deep_copy");
}

inline void deep_copy(HostMolecules& dst, const Molecules& src)
{
    dst.resize(src.size());
    dst.numLocalMolecules = src.raw()->numLocal;
    dst.numGhostMolecules = src.raw()->numGhost;
    impl::check(mrmd_molecules_download(impl::context(), src.raw(), src.size(), dst.pos.data(), dst.force.data(),
                                        dst.lambda.data(), dst.modulatedLambda.data(), dst.gradLambda.data(),
                                        dst.atomsOffset.data(), dst.numAtoms.data()),
                "deep_copy");
}
}  // namespace mrmd::data
