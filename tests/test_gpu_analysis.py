"""analysis::getKineticEnergy / getSystemMomentum / getPressure on the device,
and the same observables recorded inside the fused LJ NVE step.

Known answers: analysis/KineticEnergy.test.cpp:22-50 and
analysis/SystemMomentum.test.cpp:23-42 of the reference.  Sums over many
atoms are compared with the oracle's serial sums at 1e-12 relative (the
device sums in a fixed tree order, the oracle in index order)."""
import numpy as np
import pytest

from conftest import expect_float_eq
from test_gpu_md import fcc, mb_velocities, oracle_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


def test_kinetic_energy_kat(M):
    vel = np.array([[2.0, 0.0, 0.0], [-0.0, -8.0, -0.0], [0.0, 0.0, 16.0]])
    a = M.Atoms.from_arrays(np.zeros((3, 3)), vel=vel, mass=np.array([1.0, 2.0, 0.5]))
    expect_float_eq(M.getKineticEnergy(a), (4.0 + 2.0 * 64.0 + 0.5 * 256.0) * 0.5)
    expect_float_eq(M.getMeanKineticEnergy(a), (4.0 + 2.0 * 64.0 + 0.5 * 256.0) * 0.5 / 3)


def test_system_momentum_kat(M):
    vel = np.array([[2.0, 3.0, 4.0], [-4.0, -8.0, -16.0]])
    a = M.Atoms.from_arrays(np.zeros((2, 3)), vel=vel)
    p = M.getSystemMomentum(a)
    for got, want in zip(p, (-2.0, -5.0, -12.0)):
        expect_float_eq(got, want)


@pytest.mark.parametrize("n_local,n_ghost", [(1, 0), (1000, 300), (300_001, 40_000)])
def test_observables_vs_oracle(M, orc, n_local, n_ghost):
    rng = np.random.default_rng(n_local)
    n = n_local + n_ghost
    pos = rng.uniform(-1, 11, (n, 3))
    vel = rng.normal(0, 1.3, (n, 3))
    force = rng.normal(0, 20, (n, 3))
    mass = rng.uniform(0.5, 2.0, n)
    a = M.Atoms(n + 16)
    a.upload(n_local, n_ghost, pos=pos, vel=vel, force=force, type=np.zeros(n, dtype=np.int64), mass=mass,
             charge=np.zeros(n), relative_mass=np.ones(n))
    o = orc.Atoms(n + 16)
    o.pos[:n], o.vel[:n], o.force[:n], o.mass[:n] = pos, vel, force, mass
    o.numLocal, o.numGhost = n_local, n_ghost
    sd = M.Subdomain([0, 0, 0], [10, 9, 8], 1.0)
    osd = orc.subdomain([0, 0, 0], [10, 9, 8], 1.0)
    ke, mom, pr = M.getKineticEnergy(a), M.getSystemMomentum(a), M.getPressure(a, sd)
    np.testing.assert_allclose(ke, orc.kinetic_energy(o), rtol=1e-12)
    scale = np.abs(vel[:n_local]).sum(0)
    assert np.all(np.abs(mom - orc.system_momentum(o)) <= 1e-13 * scale)
    pscale = (np.abs(mass[:, None] * vel * vel).sum() + np.abs(force * pos).sum()) / (3 * 720.0)
    assert abs(pr - orc.pressure(o, osd)) <= 1e-13 * pscale
    # same bits on a second call (fixed reduction order)
    assert M.getKineticEnergy(a) == ke and M.getPressure(a, sd) == pr
    assert np.array_equal(M.getSystemMomentum(a), mom)


@pytest.mark.parametrize("graph", [False, True])
def test_fused_step_observables_match_oracle(M, orc, graph):
    """Kinetic energy and momentum recorded inside the FP64 step equal the
    oracle loop's getKineticEnergy / getSystemMomentum after every step, and the
    LJ energy / virial columns equal those of the stepper without recording
    (to the last bits of the energy sum)."""
    pos, L = fcc(6)
    rng = np.random.default_rng(5)
    pos = pos + rng.normal(0, 0.02, pos.shape)
    vel = mb_velocities(len(pos), 0.728, 2)
    steps = 23
    _, _, _, eo = oracle_run(orc, pos, vel, L, steps, observe=True)
    s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64, use_graph=graph, observe=True)
    rec = np.vstack([s.run_observed(10), s.run_observed(steps - 10)])
    plain = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64, use_graph=graph)
    e = np.vstack([plain.run(10), plain.run(steps - 10)])
    # (the FP64 pair kernel adds block energies with atomics: order-dependent last bits)
    np.testing.assert_allclose(rec[:, :2], e, rtol=1e-13)
    np.testing.assert_allclose(rec[:, :2], eo[:, :2], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(rec[:, 2], eo[:, 2], rtol=1e-10)
    assert np.abs(rec[:, 3:] - eo[:, 3:]).max() <= 1e-10 * np.abs(vel).sum()
    # the records agree with the state read back after the run
    _, v, _ = s.state()
    np.testing.assert_allclose(rec[-1, 2], 0.5 * (v * v).sum(), rtol=1e-12)


def test_fused_step_energy_conservation(M):
    """Total energy from the device records stays within the velocity-Verlet
    fluctuation (1e-3 per atom) over 400 steps in both forms.  The velocity
    sum stays at rounding level: in the FP64 form (half list, F_ji = -F_ij
    exactly) near 1e-12; in the mixed form each side of a pair is rounded on
    its own (full list, FP32 far pairs), a random walk of about
    sqrt(N) * 1e-7 * F_rms * dt per step."""
    pos, L = fcc(8)
    rng = np.random.default_rng(9)
    pos = pos + rng.normal(0, 0.01, pos.shape)
    vel = mb_velocities(len(pos), 0.728, 3)
    for prec, mom_tol in ((M.PREC_FP64, 1e-9), (M.PREC_MIXED, 2e-5)):
        s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=prec, observe=True)
        rec = s.run_observed(400)
        etot = rec[:, 0] + rec[:, 2]
        assert np.abs(etot - etot[0]).max() / len(pos) < 1e-3
        assert np.abs(rec[:, 3:]).max() < mom_tol
    with pytest.raises(M.MrmdError):
        M.LJSystem(pos, vel, [0, 0, 0], [L] * 3).run_observed(2)
