// The ESPResSo++ comparison of MRMD's tests/LennardJones/LennardJones.cpp:82-143,
// written against the drop-in C++ classes: a reference driver compiles
// against these headers unchanged apart from the include paths and the
// predicate objects.
//
// usage: lennard_jones_espp <positions.txt>   (32,768 lines "x y z")
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "mrmd/action/LennardJones.hpp"
#include "mrmd/communication/GhostLayer.hpp"
#include "mrmd/data/Atoms.hpp"
#include "mrmd/data/Subdomain.hpp"

using namespace mrmd;

// EXPECT_FLOAT_EQ: equal as float within 4 ULPs
static bool float_eq(double a, double b)
{
    float fa = float(a), fb = float(b);
    if (fa == fb) return true;
    int32_t ia, ib;
    std::memcpy(&ia, &fa, 4);
    std::memcpy(&ib, &fb, 4);
    auto biased = [](int32_t i) { return i < 0 ? -(int64_t)(i & 0x7fffffff) : (int64_t)i; };
    return std::llabs(biased(ia) - biased(ib)) <= 4;
}

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        std::fprintf(stderr, "usage: %s positions.txt\n", argv[0]);
        return 2;
    }
    constexpr double rc = 2.5, skin = 0.3, dt = 0.005;
    constexpr idx_t ESPP_REAL = 32768, ESPP_GHOST = 22104, ESPP_NEIGHBORS = 1310403;
    constexpr real_t ESPP_INITIAL_ENERGY = -94795.927;
    int failures = 0;
    try
    {
        auto subdomain = data::Subdomain({0_r, 0_r, 0_r}, {33.8585, 33.8585, 33.8585}, rc + skin);
        // io::restoreAtoms (io/RestoreTXT.cpp:24-74)
        data::HostAtoms h(0);
        std::ifstream fin(argv[1]);
        double x, y, z;
        while (fin >> x >> y >> z)
        {
            h.pos.push_back(x);
            h.pos.push_back(y);
            h.pos.push_back(z);
        }
        const idx_t n = idx_t(h.pos.size() / 3);
        h.vel.assign(3 * n, 0.0);
        h.force.assign(3 * n, 0.0);
        h.type.assign(n, 0);
        h.mass.assign(n, 1.0);
        h.charge.assign(n, 0.0);
        h.relativeMass.assign(n, 1.0);
        h.numLocalAtoms = n;
        data::Atoms atoms(100000);
        data::deep_copy(atoms, h);
        if (atoms.numLocalAtoms != ESPP_REAL) ++failures;

        communication::GhostLayer ghostLayer;
        ghostLayer.createGhostAtoms(atoms, subdomain);
        if (atoms.numGhostAtoms != ESPP_GHOST) ++failures;

        HalfVerletList verletList;
        verletList.build(atoms.getPos(), atoms.size(), 0, atoms.numLocalAtoms, rc + skin, 1.0,
                         subdomain.minGhostCorner.data(), subdomain.maxGhostCorner.data());
        if (verletList.numPairs() != ESPP_NEIGHBORS) ++failures;

        action::LennardJones LJ(rc, 1_r, 1_r);
        atoms.setForce(0_r);
        LJ.apply(atoms, verletList);
        const real_t e0 = LJ.getEnergy();
        if (!float_eq(e0, ESPP_INITIAL_ENERGY)) ++failures;

        action::VelocityVerlet::preForceIntegrate(atoms, dt);
        ghostLayer.updateGhostAtoms(atoms, subdomain);
        atoms.setForce(0_r);
        LJ.apply(atoms, verletList);
        ghostLayer.contributeBackGhostToReal(atoms);
        action::VelocityVerlet::postForceIntegrate(atoms, dt);
        data::HostAtoms out(0);
        data::deep_copy(out, atoms);
        double fsum[3] = {0, 0, 0};
        for (idx_t i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) fsum[d] += out.force[3 * i + d];
        // Newton's third law: the net force of the periodic system vanishes
        for (int d = 0; d < 3; ++d)
            if (std::fabs(fsum[d]) > 1e-6) ++failures;
        std::printf("{\"real\": %lld, \"ghost\": %lld, \"pairs\": %lld, \"energy\": %.9f, \"energy_after_step\": %.9f, "
                    "\"net_force\": [%.3e, %.3e, %.3e], \"failures\": %d}\n",
                    (long long)atoms.numLocalAtoms, (long long)atoms.numGhostAtoms, (long long)verletList.numPairs(), e0,
                    LJ.getEnergy(), fsum[0], fsum[1], fsum[2], failures);
    }
    catch (const Error& e)
    {
        std::fprintf(stderr, "mrmd error %d: %s\n", e.code, e.what());
        return 3;
    }
    return failures == 0 ? 0 : 1;
}
