"""The FP32 helpers of csrc/f32_round.cuh, compiled for the host:
- the integer-pipe FP64 -> FP32 rounding of the stepper's coordinate split,
  compared bit for bit with the C cast (round to nearest, ties to even) on
  random doubles of every exponent, on exact ties at the float rounding
  position and on the edges of the float range (subnormals, the largest
  float, overflow);
- the exact integer-pipe FP32 -> FP64 widening, against the C cast on every
  subnormal and one float in 97 of the rest;
- the integer-pipe coordinate split (split_bits), against the FP64
  magic-number form it replaces, bit for bit: hi from rounding x + (magic -
  origin) to the quantum grid, lo from x - (t - (magic - origin)) rounded to
  FP32 (random quanta and grid origins, exact ties, grid points, values near
  the origin and tiny values);
- the binning's FP32 floor estimate, which must give the FP64 cell formula's
  cell whenever it claims certainty (random grids and coordinates, many of
  them within 2^-50 of a cell boundary)."""
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


BINNING = r"""
#include "f32_round.cuh"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
using namespace mrmd_impl;
static int exact(double x, double mn, double rdx, int n)
{
    const double t = std::floor((x - mn) * rdx);
    return t >= 0.0 ? (t > (double)(n - 1) ? n - 1 : (int)t) : 0;
}
int main()
{
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> U(0, 1);
    long bad = 0, n = 0, open = 0;
    for (int trial = 0; trial < 500; ++trial)
    {
        const double L = std::ldexp(1.0 + U(g), (int)(U(g) * 14) - 2);
        const double mn = (U(g) - 0.5) * L * (U(g) < 0.5 ? 0.1 : 3.0);
        const int nc = std::max(1, (int)std::floor(L / (0.5 + U(g) * 3.0)));
        const double rdx = (double)nc / L;
        for (int k = 0; k < 4000; ++k)
        {
            double x;
            const double r = U(g);
            if (r < 0.6)
                x = mn + (U(g) * 1.2 - 0.1) * L;
            else if (r < 0.9)
                x = mn + (int)(U(g) * (nc + 1)) / rdx + (U(g) - 0.5) * std::ldexp(1.0, -(int)(U(g) * 50));
            else
                x = mn + (U(g) - 0.5) * 1e6;
            bool ok;
            const float t = floor_of_scaled(x, (float)mn, (float)rdx, &ok);
            ++n;
            if (!ok)
            {
                ++open;
                continue;
            }
            const int f = t >= 0.f ? (t > (float)(nc - 1) ? nc - 1 : (int)t) : 0;
            if (f != exact(x, mn, rdx, nc))
            {
                if (bad < 5) std::printf("bad x=%.17g mn=%.17g rdx=%.17g\n", x, mn, rdx);
                ++bad;
            }
        }
    }
    bool ok;
    floor_of_scaled(NAN, 0.f, 1.f, &ok);
    bad += ok;
    floor_of_scaled(INFINITY, 0.f, 1.f, &ok);
    bad += ok;
    std::printf("checked %ld open %ld mismatches %ld\n", n, open, bad);
    return bad != 0;
}
"""


def test_binning_estimate_gives_the_fp64_cell(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "binning_test.cpp"
    exe = tmp_path / "binning_test"
    src.write_text(BINNING)
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout


WIDEN = r"""
#include "f32_round.cuh"
#include <cmath>
#include <cstdio>
using namespace mrmd_impl;
int main()
{
    long bad = 0, n = 0;
    auto chk = [&](uint32_t u) {
        float f;
        std::memcpy(&f, &u, 4);
        const double a = f32_to_f64(f), b = (double)f;
        uint64_t x, y;
        std::memcpy(&x, &a, 8);
        std::memcpy(&y, &b, 8);
        ++n;
        if (x != y && !(std::isnan(a) && std::isnan(b))) ++bad;
    };
    for (uint64_t b = 0; b < (1ull << 32); b += 97) chk((uint32_t)b);
    for (uint32_t u = 0; u < 0x800000u; ++u)
    {
        chk(u);
        chk(u | 0x80000000u);
    }
    std::printf("checked %ld mismatches %ld\n", n, bad);
    return bad != 0;
}
"""


def test_f32_to_f64_matches_the_c_cast(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "widen_test.cpp"
    exe = tmp_path / "widen_test"
    src.write_text(WIDEN)
    subprocess.run([gxx, "-O2", "-std=c++17", f"-I{CSRC}", str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout


SPLIT = r"""
#include "f32_round.cuh"
#include <cmath>
#include <cstdio>
#include <random>
using namespace mrmd_impl;
static uint32_t fb(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
// the FP64 form: three additions, k from the low word of t's bits
static void fp64_form(double x, double shift, float invQ, float& h, float& l)
{
    volatile double t = x + shift;
    const double tt = t;
    uint64_t tb;
    std::memcpy(&tb, &tt, 8);
    h = (float)(int32_t)(uint32_t)tb * invQ;
    volatile double y = t - shift;
    volatile double d = x - y;
    l = (float)d;
}
int main()
{
    std::mt19937_64 g(99);
    std::uniform_real_distribution<double> U(0, 1);
    long bad = 0, n = 0;
    for (int trial = 0; trial < 4000; ++trial)
    {
        const int q = (int)(U(g) * 24) - 3;
        const double Q = std::ldexp(1.0, -q);
        const long long Ko = U(g) < 0.3 ? 0 : (long long)((U(g) - 0.5) * 2e6);
        const double o = (double)Ko * Q;
        const double shift = 6755399441055744.0 * Q - o;
        const float invQ = (float)Q;
        for (int k = 0; k < 500; ++k)
        {
            double x;
            const double r = U(g);
            if (r < 0.5)
                x = o + (U(g) * 1.1 - 0.05) * Q * 16777216.0 * U(g);
            else if (r < 0.7)
                x = o + ((double)(long long)(U(g) * 1e6) + 0.5) * Q;
            else if (r < 0.8)
                x = o + (double)(long long)(U(g) * 1e6) * Q;
            else if (r < 0.9)
                x = o + (U(g) - 0.5) * Q * std::ldexp(1.0, -(int)(U(g) * 60));
            else
                x = (U(g) - 0.5) * std::ldexp(1.0, -(int)(U(g) * 80));
            if (!(std::fabs(x - o) < Q * 16777000.0) || !(std::fabs(x / Q) < std::ldexp(1.0, 61))) continue;
            float h1, l1, h2, l2;
            fp64_form(x, shift, invQ, h1, l1);
            split_bits(x, Ko, q, invQ, h2, l2);
            ++n;
            if (fb(h1) != fb(h2) || fb(l1) != fb(l2))
            {
                if (bad < 5) std::printf("bad x=%.17g q=%d Ko=%lld\n", x, q, Ko);
                ++bad;
            }
        }
    }
    std::printf("checked %ld mismatches %ld\n", n, bad);
    return bad != 0;
}
"""


def test_integer_split_matches_the_fp64_form(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "split_test.cpp"
    exe = tmp_path / "split_test"
    src.write_text(SPLIT)
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}", str(src), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
