import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: long-running CPU test")


# EXPECT_FLOAT_EQ compares as float within 4 ULPs (googletest); this is the
# reference's tolerance for every known-answer test it ships.
def expect_float_eq(actual, expected):
    a = np.float32(actual)
    e = np.float32(expected)
    if a == e:
        return
    ai = np.array([a]).view(np.int32)[0]
    ei = np.array([e]).view(np.int32)[0]
    # map to lexicographically ordered integers (sign-magnitude -> biased)
    def biased(i):
        return (-(i & 0x7FFFFFFF)) if i < 0 else i
    assert abs(int(biased(ai)) - int(biased(ei))) <= 4, f"{actual} != {expected} (4 float ULPs)"


# Per-atom force error: max_i |F_i - R_i| / max(|R_i|, floor * rms|R|).  The
# floor only matters for atoms whose net reference force nearly vanishes
# (there the error is set by the size of the pair terms, not by |R_i|).
def per_atom_rel_err(F, R, floor=0.0):
    F = np.asarray(F, dtype=np.float64).reshape(-1, 3)
    R = np.asarray(R, dtype=np.float64).reshape(-1, 3)
    nr = np.linalg.norm(R, axis=1)
    rms = float(np.sqrt((nr ** 2).mean())) if len(nr) else 0.0
    den = np.maximum(nr, floor * rms)
    d = np.linalg.norm(F - R, axis=1)
    zero = den == 0.0
    if np.any(d[zero] != 0.0):
        return float("inf")
    den[zero] = 1.0
    return float((d / den).max()) if len(d) else 0.0


# FP64 parity bar: per atom, relative to the atom's own force (floored at
# 1e-4 of the RMS force for atoms whose force nearly cancels).
FP64_RTOL = 1e-10
FP64_FLOOR = 1e-4


def assert_fp64_forces(F, R, what=""):
    err = per_atom_rel_err(F, R, FP64_FLOOR)
    assert err <= FP64_RTOL, f"{what} per-atom FP64 force error {err:.3e} > {FP64_RTOL}"


@pytest.fixture(scope="session")
def espp():
    import json

    g = json.load(open(os.path.join(GOLDEN, "espp_golden.json")))
    pos = np.load(os.path.join(GOLDEN, "espp_positions.npz"))["milli"].astype(np.float64) / 1000.0
    return g, pos


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O

    O.set_threads(min(8, O.max_threads()))
    return O
