// A driver written with the reference's include paths (compiled with the
// drop-in's mrmd/ directory on the include path, as MRMD's own drivers are
// with MRMD's): every header a reference driver of the LJ / AdResS path
// includes resolves to the drop-in.
//
// 1. The velocity-Verlet NVE loop of examples/02_LennardJones_NVE.cpp:130-190
//    on 4,000 atoms (fcc 10^3, density 0.8442, shifted LJ, rc 2.5, skin 0.3,
//    a rebuild every 10 steps), with analysis::getKineticEnergy,
//    getSystemMomentum and getPressure checked against host sums of the
//    downloaded state.
// 2. One AdResS force evaluation (examples/04_LennardJones_IdealGas_LocalCap.cpp
//    sequence): MultiResGhostLayer, UpdateMolecules with a Slab, LJ_IdealGas,
//    ContributeMoleculeForceToAtoms, ThermodynamicForce::apply and the ghost
//    fold-back, on single-site molecules read from <dir>/molecules.txt; the
//    local atoms' forces go to <dir>/adress_forces.txt.
// 3. CoulombDSF::computeForce / computeEnergy of three pairs.
//
// usage: reference_paths <dir>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "action/ContributeMoleculeForceToAtoms.hpp"
#include "action/CoulombDSF.hpp"
#include "action/LJ_IdealGas.hpp"
#include "action/LennardJones.hpp"
#include "action/ThermodynamicForce.hpp"
#include "action/UpdateMolecules.hpp"
#include "action/VelocityVerlet.hpp"
#include "action/VelocityVerletLangevinThermostat.hpp"
#include "analysis/KineticEnergy.hpp"
#include "analysis/Pressure.hpp"
#include "analysis/SystemMomentum.hpp"
#include "communication/GhostLayer.hpp"
#include "communication/MultiResGhostLayer.hpp"
#include "data/Atoms.hpp"
#include "data/Molecules.hpp"
#include "data/Subdomain.hpp"
#include "datatypes.hpp"
#include "initialization.hpp"
#include "weighting_function/Slab.hpp"

using namespace mrmd;

// seeded uniform numbers in (0, 1) for the initial velocities (xorshift64*)
struct Uniform
{
    uint64_t s;
    double operator()()
    {
        s ^= s >> 12;
        s ^= s << 25;
        s ^= s >> 27;
        return (double((s * 2685821657736338717ull) >> 11) + 0.5) / 9007199254740992.0;
    }
};

static int nve(std::string& json)
{
    constexpr real_t rc = 2.5, skin = 0.3, dt = 0.005, rho = 0.8442, T = 0.728;
    constexpr int cells = 10, steps = 200, rebuildEvery = 10;
    const real_t a = std::cbrt(4.0 / rho), L = a * cells;
    auto subdomain = data::Subdomain({0_r, 0_r, 0_r}, {L, L, L}, rc + skin);
    const real_t basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    data::HostAtoms h(0);
    for (int x = 0; x < cells; ++x)
        for (int y = 0; y < cells; ++y)
            for (int z = 0; z < cells; ++z)
                for (const auto& b : basis)
                {
                    h.pos.push_back((x + b[0] + 0.25) * a);
                    h.pos.push_back((y + b[1] + 0.25) * a);
                    h.pos.push_back((z + b[2] + 0.25) * a);
                }
    const idx_t n = idx_t(h.pos.size() / 3);
    Uniform u{0x9e3779b97f4a7c15ull};
    h.vel.resize(3 * n);
    real_t mean[3] = {0, 0, 0};
    for (idx_t i = 0; i < 3 * n; i += 2)
    {
        const real_t r = std::sqrt(-2.0 * std::log(u())), t = 6.283185307179586 * u();
        h.vel[i] = r * std::cos(t);
        if (i + 1 < 3 * n) h.vel[i + 1] = r * std::sin(t);
    }
    for (idx_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) mean[d] += h.vel[3 * i + d] / real_t(n);
    real_t v2 = 0;
    for (idx_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d)
        {
            h.vel[3 * i + d] -= mean[d];
            v2 += h.vel[3 * i + d] * h.vel[3 * i + d];
        }
    const real_t scale = std::sqrt(3.0 * real_t(n - 1) * T / v2);
    for (auto& v : h.vel) v *= scale;
    h.force.assign(3 * n, 0.0);
    h.type.assign(n, 0);
    h.mass.assign(n, 1.0);
    h.charge.assign(n, 0.0);
    h.relativeMass.assign(n, 1.0);
    h.numLocalAtoms = n;

    data::Atoms atoms(8 * n);
    data::deep_copy(atoms, h);
    communication::GhostLayer ghostLayer;
    HalfVerletList verletList;
    action::LennardJones LJ({0_r}, {rc}, {1_r}, {1_r}, 1, true);
    auto forces = [&](bool rebuild) {
        if (rebuild)
        {
            ghostLayer.exchangeRealAtoms(atoms, subdomain);
            ghostLayer.createGhostAtoms(atoms, subdomain);
            verletList.build(atoms.getPos(), atoms.size(), 0, atoms.numLocalAtoms, rc + skin, 1.0,
                             subdomain.minGhostCorner.data(), subdomain.maxGhostCorner.data());
        }
        else
        {
            ghostLayer.updateGhostAtoms(atoms, subdomain);
        }
        atoms.setForce(0_r);
        LJ.apply(atoms, verletList);
        ghostLayer.contributeBackGhostToReal(atoms);
    };
    forces(true);
    const real_t e0 = LJ.getEnergy() + analysis::getKineticEnergy(atoms);
    real_t hostKE0 = 0;
    for (idx_t i = 0; i < 3 * n; ++i) hostKE0 += 0.5 * h.vel[i] * h.vel[i];
    const real_t ke0 = analysis::getKineticEnergy(atoms);
    for (int step = 1; step <= steps; ++step)
    {
        action::VelocityVerlet::preForceIntegrate(atoms, dt);
        forces(step % rebuildEvery == 0);
        action::VelocityVerlet::postForceIntegrate(atoms, dt);
    }
    const real_t ke = analysis::getKineticEnergy(atoms);
    const real_t e1 = LJ.getEnergy() + ke;
    const Vector3D p = analysis::getSystemMomentum(atoms);
    const real_t pressure = analysis::getPressure(atoms, subdomain);
    // the same sums on the host from the downloaded state
    data::HostAtoms out(0);
    data::deep_copy(out, atoms);
    real_t hKE = 0, hP[3] = {0, 0, 0}, hVir = 0;
    for (idx_t i = 0; i < out.numLocalAtoms; ++i)
        for (int d = 0; d < 3; ++d)
        {
            hKE += 0.5 * out.mass[i] * out.vel[3 * i + d] * out.vel[3 * i + d];
            hP[d] += out.vel[3 * i + d];
        }
    for (idx_t i = 0; i < out.numLocalAtoms + out.numGhostAtoms; ++i)
        for (int d = 0; d < 3; ++d)
            hVir += out.mass[i] * out.vel[3 * i + d] * out.vel[3 * i + d] + out.force[3 * i + d] * out.pos[3 * i + d];
    const real_t hPressure = hVir / (3.0 * L * L * L);
    char buf[1024];
    std::snprintf(buf, sizeof(buf),
                  "\"nve\": {\"atoms\": %lld, \"steps\": %d, \"e_start\": %.12e, \"e_end\": %.12e, "
                  "\"ke_start\": %.15e, \"ke_start_host\": %.15e, \"ke\": %.15e, \"ke_host\": %.15e, "
                  "\"momentum\": [%.6e, %.6e, %.6e], \"momentum_host\": [%.6e, %.6e, %.6e], "
                  "\"pressure\": %.15e, \"pressure_host\": %.15e, \"mean_ke\": %.15e, \"pairs\": %lld}",
                  (long long)n, steps, e0, e1, ke0, hostKE0, ke, hKE, p[0], p[1], p[2], hP[0], hP[1], hP[2], pressure,
                  hPressure, analysis::getMeanKineticEnergy(atoms), (long long)verletList.numPairs());
    json += buf;
    return 0;
}

static int adress(const std::string& dir, std::string& json)
{
    constexpr real_t rc = 2.5, skin = 0.3;
    const Point3D box{40_r, 12_r, 12_r};
    auto subdomain = data::Subdomain({0_r, 0_r, 0_r}, box, rc + skin);
    data::HostAtoms h(0);
    std::ifstream fin(dir + "/molecules.txt");
    double x, y, z;
    while (fin >> x >> y >> z)
    {
        h.pos.push_back(x);
        h.pos.push_back(y);
        h.pos.push_back(z);
    }
    const idx_t n = idx_t(h.pos.size() / 3);
    if (n == 0) return 1;
    h.vel.assign(3 * n, 0.0);
    h.force.assign(3 * n, 0.0);
    h.type.assign(n, 0);
    h.mass.assign(n, 1.0);
    h.charge.assign(n, 0.0);
    h.relativeMass.assign(n, 1.0);
    h.numLocalAtoms = n;
    data::HostMolecules hm(n);
    hm.pos = h.pos;
    for (idx_t i = 0; i < n; ++i)
    {
        hm.atomsOffset[i] = i;
        hm.numAtoms[i] = 1;
    }
    hm.numLocalMolecules = n;
    data::Atoms atoms(8 * n);
    data::Molecules molecules(8 * n);
    data::deep_copy(atoms, h);
    data::deep_copy(molecules, hm);

    communication::MultiResGhostLayer ghostLayer;
    weighting_function::Slab slab({20_r, 6_r, 6_r}, 10_r, 5_r, 1);
    action::LJ_IdealGas LJ(0_r, rc, 1_r, 1_r, true);
    action::ThermodynamicForce thermodynamicForce(0.5_r, subdomain, 1.2_r, 1_r);
    std::vector<real_t> table(thermodynamicForce.numBins() * thermodynamicForce.numTypes());
    for (size_t b = 0; b < table.size(); ++b) table[b] = 0.1 * std::sin(real_t(b));
    thermodynamicForce.setForce(table);
    HalfVerletList verletList;

    ghostLayer.createGhostAtoms(molecules, atoms, subdomain);
    action::UpdateMolecules::update(molecules, atoms, slab);
    verletList.build(molecules.getPos(), molecules.size(), 0, molecules.numLocalMolecules, rc + skin, 1.0,
                     subdomain.minGhostCorner.data(), subdomain.maxGhostCorner.data(), 64);
    atoms.setForce(0_r);
    molecules.setForce(0_r);
    const real_t energy = LJ.run(molecules, verletList, atoms);
    action::ContributeMoleculeForceToAtoms::update(molecules, atoms);
    thermodynamicForce.apply(atoms);
    ghostLayer.contributeBackGhostToReal(atoms);

    data::HostAtoms out(0);
    data::deep_copy(out, atoms);
    std::ofstream fo(dir + "/adress_forces.txt");
    fo.precision(17);
    for (idx_t i = 0; i < n; ++i) fo << out.force[3 * i] << ' ' << out.force[3 * i + 1] << ' ' << out.force[3 * i + 2] << '\n';
    // a Langevin thermostat object of the reference's interface (construct, set)
    action::VelocityVerletLangevinThermostat langevin(1_r, 1_r);
    langevin.set(1_r, 1_r);
    char buf[512];
    std::snprintf(buf, sizeof(buf),
                  "\"adress\": {\"molecules\": %lld, \"ghost_molecules\": %lld, \"ghost_atoms\": %lld, "
                  "\"pairs\": %lld, \"energy\": %.15e, \"bins\": %lld}",
                  (long long)n, (long long)molecules.numGhostMolecules, (long long)atoms.numGhostAtoms,
                  (long long)verletList.numPairs(), energy, (long long)thermodynamicForce.numBins());
    json += buf;
    return 0;
}

static void coulomb(std::string& json)
{
    action::impl::CoulombDSF dsf(2.5_r, 0.3_r);
    const real_t d[3] = {0.81, 2.25, 6.0}, q1[3] = {1.0, -0.5, 2.0}, q2[3] = {-1.0, 0.8, 0.3};
    json += "\"coulomb\": [";
    for (int k = 0; k < 3; ++k)
    {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s[%.17g, %.17g, %.17g, %.17g, %.17g]", k ? ", " : "", d[k], q1[k], q2[k],
                      dsf.computeForce(d[k], q1[k], q2[k]), dsf.computeEnergy(d[k], q1[k], q2[k]));
        json += buf;
    }
    json += "]";
}

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        std::fprintf(stderr, "usage: %s <dir>\n", argv[0]);
        return 2;
    }
    std::string json = "{";
    try
    {
        mrmd::initialize(argc, argv);
        if (nve(json)) return 1;
        json += ", ";
        if (adress(argv[1], json)) return 1;
        json += ", ";
        coulomb(json);
        mrmd::finalize();
    }
    catch (const Error& e)
    {
        std::fprintf(stderr, "mrmd error %d: %s\n", e.code, e.what());
        return 3;
    }
    json += "}";
    std::printf("%s\n", json.c_str());
    return 0;
}
