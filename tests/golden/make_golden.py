"""Generate the committed golden fixtures from the MRMD reference's own tests.

Run once where the MRMD source tree is available, passing its root as
``--reference``; the outputs are committed so that tests run without it.

* ``espp_positions.npz``: the 32,768 positions of
  ``tests/LennardJones/positions.txt`` (ESPResSo++ reference configuration,
  Apache-2.0, part of MRMD's test data), stored as integer thousandths
  (uint16).  Every value in the text file has at most three decimals, and
  ``q / 1000.0`` reproduces the text parse bit-for-bit (checked below).
* ``espp_golden.json``: the ESPResSo++ golden numbers, parsed from the
  constants and EXPECT lines of ``tests/LennardJones/LennardJones.cpp``.
"""
from __future__ import annotations

import argparse
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the MRMD source tree")
    args = ap.parse_args()
    src_dir = os.path.join(args.reference, "tests", "LennardJones")

    with open(os.path.join(src_dir, "positions.txt")) as f:
        pos = np.array(f.read().split(), dtype=np.float64).reshape(-1, 3)
    q = np.round(pos * 1000.0).astype(np.int64)
    assert np.all(q >= 0) and np.all(q < 65536)
    assert np.array_equal(q / 1000.0, pos), "fixture does not round-trip exactly"
    np.savez_compressed(os.path.join(HERE, "espp_positions.npz"), milli=q.astype(np.uint16))

    with open(os.path.join(src_dir, "LennardJones.cpp")) as f:
        text = f.read()

    def const(name: str) -> str:
        m = re.search(rf"{name}\s*=\s*([-0-9.]+)", text)
        assert m, name
        return m.group(1)

    m_bf = re.search(r"EXPECT_EQ\(bfAtomPairs,\s*(\d+)\)", text)
    m_box = re.search(r"\{0_r, 0_r, 0_r\},\s*\{([0-9.]+),", text)
    m_rc = re.search(r"constexpr double rc = ([0-9.]+);", text)
    m_skin = re.search(r"constexpr double skin = ([0-9.]+);", text)
    golden = {
        "source": "tests/LennardJones/LennardJones.cpp (MRMD), ESPResSo++ reference values",
        "num_real": int(const("ESPP_REAL")),
        "num_ghost": int(const("ESPP_GHOST")),
        "num_pairs": int(const("ESPP_NEIGHBORS")),
        "num_pairs_with_ghosts_bruteforce": int(m_bf.group(1)),
        "initial_energy": float(const("ESPP_INITIAL_ENERGY")),
        "box": float(m_box.group(1)),
        "rc": float(m_rc.group(1)),
        "skin": float(m_skin.group(1)),
    }
    with open(os.path.join(HERE, "espp_golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print(golden)


if __name__ == "__main__":
    main()
