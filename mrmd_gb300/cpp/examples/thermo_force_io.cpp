// MRMD's io/ThermoForce.test.cpp:11-112 (dumpSingleForce, dumpMultipleForces)
// written against the drop-in C++ classes: a table of (bin + 1)(type + 1) over
// 100 bins of x in [1, 4] is dumped, restored, and grid and forces are
// compared as EXPECT_FLOAT_EQ does.
//
// usage: thermo_force_io <directory for the two table files>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mrmd/action/AdResS.hpp"
#include "mrmd/data/Subdomain.hpp"
#include "mrmd/io/DumpThermoForce.hpp"
#include "mrmd/io/RestoreThermoForce.hpp"

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

static void fill(action::ThermodynamicForce& tf, idx_t numBins, idx_t numForces)
{
    std::vector<real_t> forces(numBins * numForces);
    for (idx_t idx = 0; idx < numBins; ++idx)
        for (idx_t jdx = 0; jdx < numForces; ++jdx)
            forces[idx * numForces + jdx] = 1_r * (real_t(idx) + 1) * (real_t(jdx) + 1);
    tf.setForce(forces);
}

static int compare(const action::ThermodynamicForce& a, const action::ThermodynamicForce& b, idx_t types)
{
    int failures = 0;
    if (a.numBins() != b.numBins() || b.numTypes() != types) return 1;
    auto g1 = a.getGrid(), g2 = b.getGrid();
    auto f1 = a.getForce(), f2 = b.getForce();
    for (idx_t i = 0; i < a.numBins(); ++i)
    {
        failures += !float_eq(g1[i], g2[i]);
        for (idx_t t = 0; t < types; ++t) failures += !float_eq(f1[i * types + t], f2[i * types + t]);
    }
    return failures;
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    const idx_t numBins = 100;
    data::Subdomain subdomain({1_r, 2_r, 3_r}, {4_r, 6_r, 8_r}, 0.5_r);
    const real_t binWidth = (subdomain.maxCorner[0] - subdomain.minCorner[0]) / real_t(numBins);
    int failures = 0;

    {  // dumpSingleForce
        action::ThermodynamicForce tf1(std::vector<real_t>{1_r}, subdomain, binWidth, std::vector<real_t>{1_r});
        fill(tf1, numBins, 1);
        io::dumpThermoForce(dir + "/dummySingleForce.txt", tf1, 0);
        auto tf2 = io::restoreThermoForce(dir + "/dummySingleForce.txt", subdomain);
        failures += compare(tf1, tf2, 1);
    }
    {  // dumpMultipleForces
        const idx_t numForces = 5;
        const std::vector<real_t> targetDensities(numForces, 1_r), modulations(numForces, 1_r);
        action::ThermodynamicForce tf1(targetDensities, subdomain, binWidth, modulations);
        fill(tf1, numBins, numForces);
        io::dumpThermoForce(dir + "/dummyMultipleForces.txt", tf1);
        auto tf2 = io::restoreThermoForce(dir + "/dummyMultipleForces.txt", subdomain, targetDensities, modulations);
        failures += compare(tf1, tf2, numForces);
    }
    std::printf("{\"failures\": %d}\n", failures);
    return failures == 0 ? 0 : 1;
}
