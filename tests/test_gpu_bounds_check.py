"""The bounds-checked debug build (libmrmd_gb300_bounds.so, -DMRMD_BOUNDS_CHECK).

The counterpart of the reference's Kokkos_ENABLE_DEBUG_BOUNDS_CHECK CI build
(.github/workflows/validate.yml:40): every kernel index into a particle, cell
or list array is tested before the access; the first violation is recorded
(file, line, index, bound), the access is skipped and the entry point returns
MRMD_ERR_BOUNDS at its next synchronisation.

The check runs in a child process that loads only the bounds-checked library
and refuses to continue unless mrmd_bounds_checked() reports it, so the bad
index below never reaches a kernel without its guard.
"""
import os
import subprocess
import sys
import textwrap

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = textwrap.dedent(r"""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, ROOT)
    import mrmd_gb300 as M
    ctx = M.default_context()
    if ctx.lib.mrmd_bounds_checked() != 1:
        print("not the bounds-checked library")
        sys.exit(3)
    L, rc, skin = 12.0, 2.5, 0.3
    rng = np.random.default_rng(5)
    pos = rng.uniform(0, L, (1000, 3))
    sd = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    a = M.Atoms.from_arrays(pos, capacity=8000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(a, sd)
    assert a.numGhostAtoms > 0
    gl.updateGhostAtoms(a, sd)          # clean: no violation
    # a host-made bad entry: the first ghost's real atom set far beyond the
    # local atoms, written into the device array from the host
    cudart = None
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            cudart = ctypes.CDLL(name)
            break
        except OSError:
            pass
    bad = np.array([1 << 30], dtype=np.int32)
    dst = ctypes.c_void_p(ctypes.cast(gl.s.correspondingRealAtom, ctypes.c_void_p).value + 4 * a.numLocalAtoms)
    assert cudart.cudaMemcpy(dst, bad.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(4), 1) == 0
    try:
        gl.updateGhostAtoms(a, sd)
    except M.MrmdError as e:
        assert e.code == -9, e
        assert "ghost.cu" in str(e) and str(1 << 30) in str(e), e
        print("reported:", e)
    else:
        print("no violation reported")
        sys.exit(4)
    # the record is cleared once reported; the context keeps working
    good = np.array([0], dtype=np.int32)
    assert cudart.cudaMemcpy(dst, good.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(4), 1) == 0
    gl.updateGhostAtoms(a, sd)
    print("ok")
""")


def test_bounds_build_reports_a_bad_ghost_index():
    from mrmd_gb300 import build as B

    B.build(bounds_check=True)
    env = dict(os.environ, MRMD_GB300_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reported: MRMD_ERR_BOUNDS" in r.stdout and r.stdout.strip().endswith("ok"), r.stdout


CLEAN = textwrap.dedent(r"""
    import sys
    import numpy as np
    sys.path.insert(0, ROOT)
    sys.path.insert(0, ROOT + "/tests")
    import mrmd_gb300 as M
    from test_gpu_md import fcc, mb_velocities
    ctx = M.default_context()
    if ctx.lib.mrmd_bounds_checked() != 1:
        print("not the bounds-checked library")
        sys.exit(3)
    pos, L = fcc(12)
    vel = mb_velocities(len(pos), 0.728, 3)
    for kw in (dict(precision=M.PREC_MIXED), dict(precision=M.PREC_MIXED, tile_build="two_kernel"),
               dict(precision=M.PREC_MIXED, gather_neighbours=True), dict(precision=M.PREC_FP64)):
        s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, **kw)
        e = s.run(45)
        assert np.all(np.isfinite(e))
        s.close()
    from adress_loop import random_system
    box = [36.0, 10.0, 10.0]
    p, v = random_system(1800, box, 5)
    for layout, prec in ((0, M.PREC_FP64), (1, M.PREC_MIXED), (2, M.PREC_MIXED)):
        b = M.BatchSystem([M.Replica(1800, [0, 0, 0], box, [18.0, 5.0, 5.0], 10.0, 77)], p, v, hybrid_diameter=5.0,
                          capping_distance=0.7842, precision=prec, list_layout=layout,
                          threads_per_row=4 if layout == 2 else 1, rebuild_interval=5, sort_every=2,
                          graph_steps=10, persistent=layout == 1)
        b.run(30)
        b.close()
    print("clean")
""")


def test_bounds_build_runs_the_steppers_clean():
    """The fused LJ stepper (both forms; the one-pass and two-kernel tile
    builds and the gather form) and the batched engine (three layouts, the
    persistent step kernel) under the bounds-checked library: every index
    stays inside its array."""
    from mrmd_gb300 import build as B

    B.build(bounds_check=True)
    env = dict(os.environ, MRMD_GB300_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CLEAN], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0 and r.stdout.strip().endswith("clean"), r.stdout + r.stderr

