"""The C++ drop-in headers (mrmd_gb300/cpp/include/mrmd/...) driving the GPU:
the reference's ESPResSo++ integration test (tests/LennardJones/LennardJones.cpp:82-143)
and io/ThermoForce.test.cpp compiled against them, and a driver that includes
every header by the reference's path."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, assert_fp64_forces

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


def test_cpp_reference_include_paths(tmp_path, orc):
    """A driver that includes every header by the reference's path
    (mrmd_gb300/cpp/examples/reference_paths.cpp): the examples/02 NVE loop
    with the analysis functions, one AdResS force evaluation in the
    examples/04 sequence against the oracle, and CoulombDSF against the
    oracle."""
    from mrmd_gb300 import build as B

    B.build()
    exe = os.path.join(ROOT, "mrmd_gb300", "_build", "reference_paths")
    assert os.path.exists(exe)
    n, box = 2500, np.array([40.0, 12.0, 12.0])
    mpos = np.random.default_rng(4).uniform(0, 1, (n, 3)) * box
    np.savetxt(tmp_path / "molecules.txt", mpos, fmt="%.17g")
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])

    # NVE: energy conserved over 200 steps; the device sums equal host sums of
    # the downloaded state
    v = out["nve"]
    assert v["atoms"] == 4000 and v["pairs"] > 0
    assert abs(v["e_end"] - v["e_start"]) <= 5e-4 * abs(v["e_start"])
    assert abs(v["ke_start"] - v["ke_start_host"]) <= 1e-12 * v["ke_start_host"]
    assert abs(v["ke"] - v["ke_host"]) <= 1e-12 * v["ke_host"]
    assert abs(v["mean_ke"] - v["ke"] / 4000) <= 1e-14 * v["ke"]
    assert np.allclose(v["momentum"], v["momentum_host"], rtol=0, atol=1e-9)
    assert np.abs(v["momentum"]).max() < 1e-6
    assert abs(v["pressure"] - v["pressure_host"]) <= 1e-10 * abs(v["pressure_host"])

    # AdResS: the oracle's examples/04 sequence on the same molecules
    rc, rlist = 2.5, 2.8
    sd = orc.subdomain([0, 0, 0], list(box), rlist)
    mo = orc.Molecules(n * 8)
    mo.pos[:n] = mpos
    mo.atomsOffset[:n] = np.arange(n)
    mo.numAtoms[:n] = 1
    mo.numLocal = n
    ao = orc.Atoms.from_positions(mpos, capacity=n * 8)
    ao.relativeMass[:n] = 1.0
    slab = orc.slab([20.0, 6.0, 6.0], 10.0, 5.0, 1)
    orc.update_molecules(mo, ao, slab)
    corr = orc.multires_create_ghosts(mo, ao, sd)
    orc.update_molecules(mo, ao, slab)
    nm = mo.numLocal + mo.numGhost
    co, no = orc.build_half_list(mo.pos, nm, 0, mo.numLocal, rlist, sd.minGhostCorner, sd.maxGhostCorner, 1.0, 96)
    ljo = orc.LJIdealGas(0.0, rc, 1.0, 1.0, True)
    ao.force[:] = 0
    mo.force[:] = 0
    E = ljo.run(mo, co, no, ao)
    orc.contribute_molecule_force(mo, ao)
    tf = orc.ThermodynamicForce([0.5], sd, 1.2, [1.0])
    tf.force[:, 0] = 0.1 * np.sin(np.arange(tf.force.shape[0]))
    tf.apply(ao)
    orc.ghost_to_real(ao, corr)
    a = out["adress"]
    assert a["molecules"] == n and a["ghost_molecules"] == mo.numGhost and a["ghost_atoms"] == ao.numGhost
    assert a["pairs"] == int(co.sum()) and a["bins"] == tf.force.shape[0]
    assert abs(a["energy"] - E) <= 1e-10 * max(abs(E), 1.0)
    f = np.loadtxt(tmp_path / "adress_forces.txt")
    assert_fp64_forces(f, ao.force[:n], "drop-in AdResS step")

    # CoulombDSF pair function (device exp against the host's: last bits)
    o = orc.CoulombDSF(2.5, 0.3)
    for d, q1, q2, fg, eg in out["coulomb"]:
        s = 138.9 * abs(q1 * q2)
        assert abs(fg - o.computeForce(d, q1, q2)) <= 1e-13 * (abs(o.computeForce(d, q1, q2)) + s / d)
        assert abs(eg - o.computeEnergy(d, q1, q2)) <= 1e-13 * s / np.sqrt(d)
