"""impl::CoulombDSF (action/CoulombDSF.hpp:39-83) and its half-list pair force.

Known answers: action/CoulombDSF.test.cpp:23-117 of the reference: energy and
force against the closed form with the exact erfc (relative error below 1e-5
and 1e-4, the approximate erfc's accuracy), charge symmetry (EXPECT_FLOAT_EQ)
and a vanishing force at the cutoff.  The oracle is pinned by them on the CPU;
the device pair function and pair force are compared with the oracle."""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import expect_float_eq

INV_SQRTPI = 1.0 / math.sqrt(math.pi)


def energy_exact(r, q1, q2, alpha, rc):
    # CoulombDSF.test.cpp:31-42
    prefac = 138.935458 * q1 * q2
    b = math.erfc(alpha * r) / r - math.erfc(alpha * rc) / rc
    b += (math.erfc(alpha * rc) / (rc * rc)
          + 2 * alpha * INV_SQRTPI * math.exp(-alpha * alpha * rc * rc) / rc) * (r - rc)
    return prefac * b


def force_exact(r, q1, q2, alpha, rc):
    # CoulombDSF.test.cpp:44-59
    prefac = 138.935458 * q1 * q2
    b = math.erfc(alpha * r) / (r * r) + 2 * alpha * INV_SQRTPI * math.exp(-alpha * alpha * r * r) / r
    b -= math.erfc(alpha * rc) / (rc * rc) + 2 * alpha * INV_SQRTPI * math.exp(-alpha * alpha * rc * rc) / rc
    return prefac * b / r


def kat_check(make):
    """The four tests of CoulombDSF.test.cpp for a factory make(rc, alpha)
    returning an object with computeForce / computeEnergy (vectorised or not)."""
    rc, alpha, q1, q2 = 5.0, 0.1, 1.2, -1.3
    c = make(rc, alpha)
    xs = np.arange(1e-8, rc - 1.0, 0.01)
    got = np.asarray(c.computeEnergy(xs * xs, q1, q2))
    want = np.array([energy_exact(x, q1, q2, alpha, rc) for x in xs])
    assert np.all(np.abs((got - want) / want) < 1e-5)
    xs = np.arange(1e-8, rc, 0.01)
    got = np.asarray(c.computeForce(xs * xs, q1, q2))
    want = np.array([force_exact(x, q1, q2, alpha, rc) for x in xs])
    assert np.all(np.abs((got - want) / want) < 1e-4)
    c = make(1.0, 0.1)
    f = lambda a, b: float(np.asarray(c.computeForce(1.0, a, b)))  # noqa: E731
    expect_float_eq(f(1, 1), f(-1, -1))
    expect_float_eq(f(1, -1), f(-1, 1))
    expect_float_eq(f(1, 1), -f(1, -1))
    c = make(1.5, 0.1)
    assert abs(float(np.asarray(c.computeForce(1.5 * 1.5, 1, 1)))) < 1e-5


class _VecOracle:
    def __init__(self, orc, rc, alpha):
        self.c = orc.CoulombDSF(rc, alpha)

    def computeEnergy(self, d, q1, q2):
        return np.vectorize(lambda x: self.c.computeEnergy(x, q1, q2))(d)

    def computeForce(self, d, q1, q2):
        return np.vectorize(lambda x: self.c.computeForce(x, q1, q2))(d)


def test_oracle_kats(orc):
    kat_check(lambda rc, alpha: _VecOracle(orc, rc, alpha))


def test_approx_erfc_accuracy(orc):
    """util::approxErfc (Abramowitz & Stegun 7.1.26): |error| <= 1.5e-7."""
    for x in np.linspace(1e-6, 6, 601):
        assert abs(orc.approx_erfc(x) - math.erfc(x)) <= 1.5e-7


def test_library_shifts_match_oracle(orc):
    """The constructor's shifts are host arithmetic: bit-identical."""
    from mrmd_gb300 import _abi
    for rc, alpha in ((5.0, 0.1), (1.0, 0.1), (1.5, 0.1), (9.0, 0.35)):
        p = _abi.CoulombDSFS()
        assert _abi.lib().mrmd_coulomb_dsf_init(C.byref(p), rc, alpha) == 0
        o = orc.CoulombDSF(rc, alpha).c
        for k in ("alpha", "rc", "rcSqr", "forceShift", "energyShift"):
            assert getattr(p, k) == getattr(o, k), k
    p = _abi.CoulombDSFS()
    assert _abi.lib().mrmd_coulomb_dsf_init(C.byref(p), 0.0, 0.1) != 0


# ------------------------------------------------------------------- GPU ---

@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


@pytest.mark.gpu
def test_device_kats(M):
    kat_check(lambda rc, alpha: M.CoulombDSF(rc, alpha))


@pytest.mark.gpu
def test_device_pair_function_vs_oracle(M, orc):
    rng = np.random.default_rng(4)
    rc, alpha = 9.0, 0.35
    d = rng.uniform(0.3, rc, 20000) ** 2
    q1, q2 = rng.uniform(-1.5, 1.5, (2, d.size))
    f, e = M.CoulombDSF(rc, alpha)._eval(d, q1, q2)
    o = orc.CoulombDSF(rc, alpha)
    fo = np.array([o.computeForce(*t) for t in zip(d, q1, q2)])
    eo = np.array([o.computeEnergy(*t) for t in zip(d, q1, q2)])
    # device exp() and the host's differ in the last bit at most
    assert np.all(np.abs(f - fo) <= 1e-13 * np.abs(fo) + 1e-13 * np.abs(138.9 * q1 * q2) / d)
    assert np.all(np.abs(e - eo) <= 1e-13 * np.abs(138.9 * q1 * q2) / np.sqrt(d))


@pytest.mark.gpu
@pytest.mark.parametrize("n,L,rc", [(1500, 12.0, 3.0), (6000, 18.0, 4.5)])
def test_device_pair_force_vs_oracle(M, orc, n, L, rc):
    rng = np.random.default_rng(n)
    pos = rng.uniform(0, L, (n, 3))
    q = rng.choice([-1.0, 1.0], n) * rng.uniform(0.3, 1.0, n)
    skin, alpha = 0.3, 0.25
    sd_o = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    ao = orc.Atoms.from_positions(pos, capacity=12 * n)
    ao.charge[:n] = q
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 256)
    ao.force[:] = 0
    Eo, Wo = orc.CoulombDSF(rc, alpha).apply(ao, co, no)
    orc.ghost_to_real(ao, corr)

    sd_g = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    ag = M.Atoms(12 * n)
    ag.upload(n, 0, pos=pos, vel=np.zeros((n, 3)), force=np.zeros((n, 3)), type=np.zeros(n, dtype=np.int64),
              mass=np.ones(n), charge=q, relative_mass=np.ones(n))
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 256)
    ag.setForce(0.0)
    c = M.CoulombDSF(rc, alpha)
    Eg = c.apply(ag, vl)
    gl.contributeBackGhostToReal(ag)
    Fg = ag.getForce(n)
    scale = np.abs(ao.force[:n]).max()
    assert np.abs(Fg - ao.force[:n]).max() <= 1e-10 * scale
    assert abs(Eg - Eo) <= 1e-10 * max(abs(Eo), 1.0)
    assert abs(c.getVirial() - Wo) <= 1e-10 * max(abs(Wo), 1.0)
    # Newton's third law over the whole system
    assert np.abs(Fg.sum(0)).max() <= 1e-9 * scale
