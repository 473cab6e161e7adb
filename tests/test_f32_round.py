"""The integer-pipe FP64 -> FP32 rounding of the stepper's coordinate split
(csrc/f32_round.cuh), compiled for the host and compared bit for bit with
the C cast (round to nearest, ties to even) on random doubles of every
exponent, on exact ties at the float rounding position, and on the edges of
the float range (subnormals, the largest float, overflow)."""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mrmd_gb300", "csrc")

DRIVER = r"""
#include "f32_round.cuh"
#include <cmath>
#include <cstdio>
#include <random>
using namespace mrmd_impl;
static uint32_t fb(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
int main()
{
    std::mt19937_64 g(12345);
    long bad = 0, n = 0;
    auto chk = [&](double d) {
        const float a = f64_to_f32_rn(d), b = (float)d;
        ++n;
        if (fb(a) != fb(b) && !(std::isnan(a) && std::isnan(b)))
        {
            if (bad < 5) std::printf("mismatch %.17g: %08x vs %08x\n", d, fb(a), fb(b));
            ++bad;
        }
    };
    for (long i = 0; i < 2000000; ++i)
    {
        const uint64_t b = g();
        double d;
        std::memcpy(&d, &b, 8);
        chk(d);
    }
    for (int e = -160; e <= 130; ++e)
        for (int k = 0; k < 2000; ++k)
        {
            double d = std::ldexp(1.0 + (double)(g() >> 12) / 4503599627370496.0, e);
            chk(d);
            chk(-d);
            uint64_t b;
            std::memcpy(&b, &d, 8);
            b = (b & ~0x1fffffffull) | 0x10000000ull;  // exactly half a float ulp below
            std::memcpy(&d, &b, 8);
            chk(d);
            chk(-d);
        }
    const double edges[] = {0.0, -0.0, INFINITY, -INFINITY, 3.4028235677973366e38, 3.4028234663852886e38,
                            1.401298464324817e-45, 7.006492321624085e-46, 7.006492321624087e-46,
                            1.1754942106924411e-38, 5e-324, 1e-300, 2.2250738585072014e-308};
    for (double d : edges)
    {
        chk(d);
        chk(-d);
    }
    std::printf("checked %ld mismatches %ld\n", n, bad);
    return bad != 0;
}
"""


def test_f64_to_f32_matches_the_c_cast(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "f32_round_test.cpp"
    exe = tmp_path / "f32_round_test"
    src.write_text(DRIVER)
    subprocess.run([gxx, "-O2", "-std=c++17", f"-I{CSRC}", str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
