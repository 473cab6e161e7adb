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
