// Drop-in data::Molecules / data::HostMolecules (data/Molecules.hpp:27-176):
// device storage through the C ABI and a host mirror, moved by deep_copy.
#pragma once

#include <vector>

#include "../datatypes.hpp"

namespace mrmd::data
{
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
    explicit Molecules(idx_t n) { gb300::check(mrmd_molecules_alloc(gb300::context(), &m_, n), "Molecules"); }
    ~Molecules() { mrmd_molecules_free(gb300::context(), &m_); }
    Molecules(const Molecules&) = delete;
    Molecules& operator=(const Molecules&) = delete;

    double* getPos() const { return m_.pos; }
    void setForce(const real_t& val)
    {
        gb300::check(mrmd_molecules_set_force(gb300::context(), &m_, size(), val), "setForce");
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
    gb300::check(mrmd_molecules_upload(gb300::context(), dst.raw(), src.numLocalMolecules, src.numGhostMolecules,
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
    gb300::check(mrmd_molecules_download(gb300::context(), src.raw(), src.size(), dst.pos.data(), dst.force.data(),
                                        dst.lambda.data(), dst.modulatedLambda.data(), dst.gradLambda.data(),
                                        dst.atomsOffset.data(), dst.numAtoms.data()),
                "deep_copy");
}
}  // namespace mrmd::data
