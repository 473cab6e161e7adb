"""The 4,000,000-atom LJ fluid of the precision study at full size, through
size-independent properties: mixed-form forces within 1e-6 of the FP64 form's
per atom (floored at 0.1 of the RMS force), energies and virials within 1e-9, Newton's
third law (the FP64 half-list forces sum to zero up to rounding), and both
lists holding every pair within the list radius (the full list has each pair
twice: local-local pairs from both ends, local-ghost pairs once per end that
is local)."""
import numpy as np
import pytest

from conftest import per_atom_rel_err

from test_gpu_md import fcc, mb_velocities

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


def test_lj_4m_mixed_vs_fp64(M):
    pos, L = fcc(100)
    n = len(pos)
    assert n == 4_000_000
    vel = mb_velocities(n, 0.728, 1000)
    ref = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64)
    ref.run(20, energies=False)
    p, v, _ = ref.state()
    mix = M.LJSystem(p, v, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED)
    ref.set_state(p, v)
    er, wr = ref.eval_forces()
    em, wm = mix.eval_forces()
    _, _, fr = ref.state()
    _, _, fm = mix.state()
    rms = float(np.sqrt((fr * fr).sum(1).mean()))
    err = float(np.linalg.norm(fm - fr, axis=1).max()) / rms
    assert err < 1e-6, err
    assert per_atom_rel_err(fm, fr, 0.1) < 1e-6
    assert abs(em - er) <= 1e-9 * abs(er)
    assert abs(wm - wr) <= 1e-9 * abs(wr)
    # Newton's third law: pair forces cancel (rounding of 4 M sums only)
    assert np.abs(fr.sum(0)).max() <= 1e-9 * rms * n
    half, full = ref.stats()["pairs"], mix.stats()["pairs"]
    assert 1.9 * half < full < 2.0 * half + 1
