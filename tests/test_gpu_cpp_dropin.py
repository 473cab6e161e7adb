"""The C++ drop-in headers (mrmd_gb300/cpp/include/mrmd/...) driving the GPU:
the reference's ESPResSo++ integration test (tests/LennardJones/LennardJones.cpp:82-143)
compiled against them."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cpp_espp_driver(tmp_path, espp):
    from mrmd_gb300 import build as B

    B.build()
    exe = os.path.join(ROOT, "mrmd_gb300", "_build", "lennard_jones_espp")
    assert os.path.exists(exe)
    g, pos = espp
    f = tmp_path / "positions.txt"
    np.savetxt(f, pos, fmt="%.3f")
    r = subprocess.run([exe, str(f)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["real"] == g["num_real"]
    assert out["ghost"] == g["num_ghost"]
    assert out["pairs"] == g["num_pairs"]
    assert out["failures"] == 0


def test_cpp_thermo_force_io(tmp_path):
    """io/ThermoForce.test.cpp (dumpSingleForce, dumpMultipleForces) through
    the drop-in io::dumpThermoForce / io::restoreThermoForce."""
    from mrmd_gb300 import build as B

    B.build()
    exe = os.path.join(ROOT, "mrmd_gb300", "_build", "thermo_force_io")
    assert os.path.exists(exe)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1])["failures"] == 0
    assert (tmp_path / "dummyMultipleForces.txt").read_text().count("\n") == 6
