"""The CPU oracle against the reference's own golden vectors and known-answer
tests.  These pin the oracle before it is trusted as the GPU checker."""
import numpy as np
import pytest

from conftest import expect_float_eq


# ------------------------------------------------------------------ ESPP ---

def test_espp_golden_counts_and_energy(orc, espp):
    """tests/LennardJones/LennardJones.cpp:82-128"""
    g, pos = espp
    L, rc, skin = g["box"], g["rc"], g["skin"]
    sd = orc.subdomain([0, 0, 0], [L, L, L], rc + skin)
    at = orc.Atoms.from_positions(pos, capacity=60000)
    assert at.numLocal == g["num_real"]
    assert orc.count_within(at.pos, at.numLocal, at.numLocal, rc + skin, [L] * 3, True) == g["num_pairs"]
    corr = orc.create_ghosts(at, sd)
    assert at.numGhost == g["num_ghost"]
    assert orc.count_within(at.pos, at.numLocal, at.n, rc + skin, [L] * 3, False) == \
        g["num_pairs_with_ghosts_bruteforce"]
    counts, nbrs = orc.build_half_list(at.pos, at.n, 0, at.numLocal, rc + skin,
                                       sd.minGhostCorner, sd.maxGhostCorner, 1.0, 60)
    assert counts.sum() == g["num_pairs"]
    tab = orc.lj_table(0.0, rc, 1.0, 1.0, 1, False)
    E, _ = orc.lj_apply(tab, rc * rc, at, counts, nbrs)
    expect_float_eq(E, g["initial_energy"])

    # pair identity: every list pair is a distinct periodic pair within r_list,
    # and there are as many as the brute-force periodic count -> same set.
    keys = orc.canonical_pairs(counts, nbrs, corr, at.numLocal)
    assert len(np.unique(keys)) == g["num_pairs"]
    a, b = keys >> 32, keys & 0xFFFFFFFF
    d = pos[a] - pos[b]
    d -= L * np.round(d / L)
    assert np.all((d * d).sum(1) <= (rc + skin) ** 2)


# ------------------------------------------------------------ LJ closed form -

def test_lj_explicit_comparison(orc):
    """action/LennardJones.test.cpp:46-81"""
    epsilon, sigma = 2.0, 3.01
    rc = 2.5 * sigma
    cap = 0.1
    cutoff_pot = 4 * epsilon * ((sigma / rc) ** 12 - (sigma / rc) ** 6)
    tab = orc.lj_table(cap, rc, sigma, epsilon, 1, True)
    delta = 0.1
    start = cap + delta
    for idx in range(100):
        x = start + idx * delta
        ff, e = orc.lj_force_energy(tab, x * x)
        pot = 4 * epsilon * ((sigma / x) ** 12 - (sigma / x) ** 6) - cutoff_pot
        expect_float_eq(e, pot)
        force = 4 * epsilon * (-12 * (sigma / x) ** 12 + 6 * (sigma / x) ** 6) * x / (x * x)
        expect_float_eq(-x * ff, force)


def test_lj_capping_constant_force(orc):
    """Inside the capping distance |F| = |F(r_cap)| (action/LennardJones.hpp:70-77)."""
    tab = orc.lj_table(0.7, 2.5, 1.0, 1.0, 1, True)
    ffc, _ = orc.lj_force_energy(tab, 0.7 ** 2)
    for r in (0.1, 0.3, 0.5, 0.69):
        ff, e = orc.lj_force_energy(tab, r * r)
        assert abs(ff * r - ffc * 0.7) <= 1e-12 * abs(ffc * 0.7)
    # |F(r_cap)| = 4662.7 for r_cap = 0.7 (example 04 setting)
    assert abs(ffc * 0.7 - 4662.7) < 0.05


# -------------------------------------------------------------- integrators -

def single_atom(orc):
    """test/SingleAtom.hpp:28-60"""
    a = orc.Atoms(1)
    a.pos[0] = (2, 3, 4)
    a.vel[0] = (7, 5, 3)
    a.force[0] = (9, 7, 8)
    a.mass[0] = 1.5
    a.charge[0] = 0.5
    a.numLocal = 1
    return a


def test_vv_pre(orc):
    """action/VelocityVerlet.test.cpp:27-48"""
    a = single_atom(orc)
    orc.vv_pre(a, 4.0)
    for got, exp in zip(a.force[0], (9, 7, 8)):
        expect_float_eq(got, exp)
    for got, exp in zip(a.vel[0], (19, 14.333333, 13.666667)):
        expect_float_eq(got, exp)
    for got, exp in zip(a.pos[0], (78, 60.333332, 58.666668)):
        expect_float_eq(got, exp)


def test_vv_post(orc):
    """action/VelocityVerlet.test.cpp:50-71"""
    a = single_atom(orc)
    orc.vv_post(a, 4.0)
    for got, exp in zip(a.vel[0], (19, 14.333333, 13.666667)):
        expect_float_eq(got, exp)
    for got, exp in zip(a.pos[0], (2, 3, 4)):
        expect_float_eq(got, exp)


def test_philox_known_answer(orc):
    """Philox4x32-10 known-answer vectors published with Random123 (kat_vectors):
    counter 0 / key 0 and counter all-ones / key all-ones."""
    assert orc.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == \
        [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def test_langevin_statistics(orc):
    """Ornstein-Uhlenbeck step drives an ideal gas to the target temperature
    (tests/LangevinThermostat/LangevinThermostat.cpp:82-136 checks T within 0.01
    for 100k atoms; smaller system and looser band here)."""
    n = 20000
    a = orc.Atoms(n)
    rng = np.random.default_rng(1)
    a.pos[:n] = rng.uniform(0, 10, (n, 3))
    a.mass[:n] = 1.0
    a.numLocal = n
    for step in range(400):
        orc.langevin_pre(a, 0.01, 1.0, 1.5, 1234, step)
        orc.vv_post(a, 0.01)
    T = (a.vel[:n] ** 2).sum() / (3 * n)
    assert abs(T - 1.5) < 0.05


# ------------------------------------------------------------- ghost layer -

def grid27(orc):
    """communication/GhostExchange.test.cpp:67-93"""
    pts = [(x + 0.5, y + 0.5, z + 0.5) for x in range(3) for y in range(3) for z in range(3)]
    return orc.Atoms.from_positions(np.array(pts), capacity=200)


def test_ghost_exchange_xyz(orc):
    """communication/GhostExchange.test.cpp:119-153"""
    sd = orc.subdomain([0, 0, 0], [3, 3, 3], 0.7)
    a = grid27(orc)
    assert orc.count_within(a.pos, 27, 27, 1.1, [3, 3, 3], False) == 12 * 3 + 9 * 2
    assert orc.count_within(a.pos, 27, 27, 1.1, [3, 3, 3], True) == 27 * 6 // 2
    corr = orc.create_ghosts(a, sd)
    assert a.numGhost == 98
    assert np.all(corr[:27] == -1)
    assert np.all(corr[27:a.n] < 27) and np.all(corr[27:a.n] >= 0)
    assert orc.count_within(a.pos, 27, a.n, 1.1, [3, 3, 3], False) == 108


def test_update_ghosts_and_reduce(orc):
    """UpdateGhostAtoms.cpp:31-68 / AccumulateForce.cpp:25-47: ghosts follow
    real atoms with the periodic shift; ghost forces fold back and are zeroed."""
    sd = orc.subdomain([0, 0, 0], [3, 3, 3], 0.7)
    a = grid27(orc)
    corr = orc.create_ghosts(a, sd)
    shift0 = a.pos[27:a.n] - a.pos[corr[27:a.n]]
    a.pos[:27] += 0.01
    orc.update_ghosts(a, corr, sd)
    np.testing.assert_array_equal(a.pos[27:a.n] - a.pos[corr[27:a.n]], np.round(shift0))
    a.force[27:a.n] = 1.0
    orc.ghost_to_real(a, corr)
    assert np.all(a.force[27:a.n] == 0)
    np.testing.assert_array_equal(a.force[:27, 0], np.bincount(corr[27:a.n], minlength=27))


def test_map_into_domain(orc):
    """communication/PeriodicMapping.test.cpp:46-83 behaviour: wrap into [min,max)."""
    sd = orc.subdomain([0, 0, 0], [3, 3, 3], 0.7)
    a = orc.Atoms.from_positions(np.array([[-0.5, 3.5, 1.0], [3.0, -3.0, 2.999], [3.5, 0.0, -1e-17]]))
    orc.map_into_domain(a, sd)
    assert np.all(a.pos[:3] >= 0) and np.all(a.pos[:3] < 3)
    np.testing.assert_allclose(a.pos[0], [2.5, 0.5, 1.0])
    # -1e-17 + 3 rounds to 3.0 == max, which the reference maps to min (PeriodicMapping.cpp:47-50)
    assert a.pos[2, 2] == 0.0


# ------------------------------------------------------ histograms and TF -

def test_multihistogram_ops(orc):
    """data/MultiHistogram.test.cpp:25-293"""
    h = orc.Histogram(0, 10, 10, 2)
    assert h.get_bin(-0.5) == -1 and h.get_bin(0.5) == 0 and h.get_bin(5.5) == 5
    assert h.get_bin(10.5) == -1
    expect_float_eq(h.bin_position(0), 0.5)
    for i in range(10):
        assert h.get_bin(h.bin_position(i)) == i
    s = orc.Histogram(0, 10, 10, 2)
    s.data[:, 0] = np.arange(10)
    s.data[:, 1] = 10 - np.arange(10)
    s.make_symmetric()
    assert np.allclose(s.data[:, 0], 4.5) and np.allclose(s.data[:, 1], 5.5)
    g = orc.Histogram(0, 10, 10, 3)
    g.data[:, 0] = 1
    g.data[:, 1] = np.arange(10)
    g.data[:, 2] = 10 - np.arange(10)
    gr = g.gradient(False)
    assert np.allclose(gr.data, [[0, 1, -1]] * 10)
    sm = orc.Histogram(0, 10, 11, 2)
    sm.data[5] = (10, 5)
    out = sm.smoothen(1.0, 3.0)
    for i in range(1, 6):
        expect_float_eq(out.data[5 - i, 0], out.data[5 + i, 0])
        expect_float_eq(out.data[5 - i, 1], out.data[5 + i, 1])
    c = orc.Histogram(0, 10, 11, 1)
    c.data[:] = 2.0
    for v in c.smoothen(1.0, 3.0).data[:, 0]:
        expect_float_eq(v, 2.0)
    r = orc.Histogram(0, 10, 11, 2)
    r.data[:] = np.arange(11)[:, None] * 10 + np.arange(2)[None, :]
    r.replace_if(orc.pred(orc.PRED_IN_OPEN_INTERVAL, 0, 0, -np.inf, 5.0), -1.0)
    for i in range(11):
        if r.bin_position(i) < 5:
            assert np.all(r.data[i] == -1)
        else:
            assert np.all(r.data[i] == [i * 10, i * 10 + 1])


def test_axial_density_profile(orc):
    """analysis/AxialDensityProfile.test.cpp:27-71"""
    xs, ts = [], []
    for i in range(10):
        for _ in range(i + 1):
            xs += [i + 0.5, 10 - (i + 0.5)]
            ts += [0, 1]
    a = orc.Atoms.from_positions(np.stack([xs, np.zeros(len(xs)), np.zeros(len(xs))], 1))
    a.type[: len(ts)] = ts
    h = orc.axial_density_profile(a, 2, 0, 10, 10)
    for i in range(10):
        expect_float_eq(h.data[i, 0], i + 1)
        expect_float_eq(h.data[i, 1], 11 - (i + 1))


def tf_fixture(orc):
    """action/ThermodynamicForce.test.cpp:79-94"""
    sd = orc.subdomain([0, 0, 0], [10, 1, 1], 1.0)
    tf = orc.ThermodynamicForce([1.0], sd, 1.0, [1.0])
    tf.force[:, 0] = np.arange(tf.force.shape[0])
    return tf


def uniform_atoms(orc):
    """getAtoms, ThermodynamicForce.test.cpp:42-54"""
    x = np.arange(100) / 10.0
    return orc.Atoms.from_positions(np.stack([x, 0 * x, 0 * x], 1))


def nonuniform_atoms(orc):
    """getAtomsNonuniform, ThermodynamicForce.test.cpp:56-77"""
    xs = [idx + 0.5 for idx in range(10) for _ in range(idx)]
    return orc.Atoms.from_positions(np.stack([xs, np.zeros(45), np.zeros(45)], 1))


def test_tf_sample_and_apply(orc):
    """ThermodynamicForce.test.cpp:96-198"""
    tf = tf_fixture(orc)
    a = uniform_atoms(orc)
    tf.sample(a)
    assert np.all(tf.density[:, 0] == 10)
    tf2 = tf_fixture(orc)
    tf2.sample(nonuniform_atoms(orc))
    assert np.all(tf2.density[:, 0] == np.arange(10))
    a = uniform_atoms(orc)
    tf.apply(a)
    np.testing.assert_array_equal(a.force[:100, 0], np.floor(a.pos[:100, 0]))
    a = uniform_atoms(orc)
    tf.apply(a, orc.pred(orc.PRED_IN_OPEN_INTERVAL, 0, 0, 0.5, 4.5))
    x = a.pos[:100, 0]
    sel = (x > 0.5) & (x < 4.5)
    np.testing.assert_array_equal(a.force[:100, 0][sel], np.floor(x[sel]))
    assert np.all(a.force[:100, 0][~sel] == 0)
    a = uniform_atoms(orc)
    tf.apply_interpolated(a, orc.pred(orc.PRED_IN_OPEN_INTERVAL, 0, 0, 0.5, 4.5))
    for xi, fi, s in zip(x, a.force[:100, 0], sel):
        if s:
            expect_float_eq(fi, xi - 0.5)
        else:
            assert fi == 0


def test_tf_update(orc):
    """ThermodynamicForce.test.cpp:200-245"""
    tf = tf_fixture(orc)
    tf.sample(nonuniform_atoms(orc))
    assert tf.update(1.0, 0.0) == 0
    for i in range(10):
        expect_float_eq(tf.force[i, 0], i - 1.0)
    assert tf.samples == 0 and np.all(tf.density == 0)
    tf = tf_fixture(orc)
    tf.sample(nonuniform_atoms(orc))
    tf.update(1.0, 0.0, orc.pred(orc.PRED_IN_OPEN_INTERVAL, 0, 0, 0.51, 4.49))
    for i in range(10):
        x = i + 0.5
        expect_float_eq(tf.force[i, 0], i - 1.0 if 0.51 < x < 4.49 else float(i))


# ------------------------------------------------------------------ AdResS -

def test_slab_regions_and_boundaries(orc):
    """weighting_function/Slab.test.cpp:23-80"""
    s = orc.slab([2, 3, 4], 2.0, 2.0, 2)
    w_prev = orc.slab_eval(s, 2.0)[1]
    x = 2.0
    for _ in range(60):
        w = orc.slab_eval(s, x)[1]
        assert w <= w_prev
        w_prev = w
        x += 0.1
    expect_float_eq(orc.slab_eval(s, 2.9)[1], 1.0)
    expect_float_eq(orc.slab_eval(s, 5.1)[1], 0.0)
    # gradient is d(modulatedLambda)/dx (central difference check in HY)
    for x in (3.2, 3.7, 4.4):
        h = 1e-6
        fd = (orc.slab_eval(s, x + h)[1] - orc.slab_eval(s, x - h)[1]) / (2 * h)
        assert abs(fd - orc.slab_eval(s, x)[2]) < 1e-6


def diamond(orc):
    """test/DiamondFixture.hpp:26-131"""
    m = orc.Molecules(2)
    m.atomsOffset[:2] = (0, 2)
    m.numAtoms[:2] = (2, 2)
    m.numLocal = 2
    a = orc.Atoms.from_positions(np.array([[1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0.0]]))
    a.mass[:4] = (1, 3, 1, 3)
    a.relativeMass[:4] = (0.25, 0.75, 0.25, 0.75)
    return m, a


def test_update_molecules_com(orc):
    """action/UpdateMolecules.test.cpp:43-60 (COM part; lambda via Slab)"""
    m, a = diamond(orc)
    orc.update_molecules(m, a, orc.slab([0, 0, 0], 10, 1, 1))
    for got, exp in zip(m.pos[0], (0.25, 0.75, 0)):
        expect_float_eq(got, exp)
    for got, exp in zip(m.pos[1], (-0.25, -0.75, 0)):
        expect_float_eq(got, exp)
    assert m.modulatedLambda[0] == 1.0


def test_contribute_molecule_force(orc):
    """action/ContributeMoleculeForceToAtoms.test.cpp:27-51"""
    m, a = diamond(orc)
    m.force[0] = (5, 6, 7)
    orc.contribute_molecule_force(m, a)
    np.testing.assert_allclose(a.force[0], np.array([5, 6, 7]) * 0.25)
    np.testing.assert_allclose(a.force[1], np.array([5, 6, 7]) * 0.75)


def ljig_fixture(orc, lam):
    """action/LJ_IdealGas.test.cpp:34-138: two 2-atom molecules, list with
    cutoff 2 on [-1,1]^3."""
    m = orc.Molecules(2)
    m.pos[:2] = [[-0.5, 0, 0], [0.5, 0, 0]]
    m.atomsOffset[:2] = (0, 2)
    m.numAtoms[:2] = (2, 2)
    m.numLocal = 2
    m.modulatedLambda[:2] = lam
    a = orc.Atoms.from_positions(np.array([[-0.5, -0.5, 0], [-0.5, 0.5, 0], [0.5, -0.5, 0],
                                           [0.5, 0.5, 0]]))
    a.relativeMass[:4] = 0.5
    counts, nbrs = orc.build_half_list(m.pos, 2, 0, 2, 2.0, [-1, -1, -1], [1, 1, 1], 1.0, 4)
    return m, a, counts, nbrs


@pytest.mark.parametrize("lam,scale", [(0.0, None), (0.5, 0.5), (1.0, 1.0)])
def test_lj_ideal_gas_kat(orc, lam, scale):
    """action/LJ_IdealGas.test.cpp:140-220 (CG / HY / AT)"""
    m, a, counts, nbrs = ljig_fixture(orc, lam)
    sigma = 0.9
    lj = orc.LJIdealGas(0.0, 2.5 * sigma, sigma, 2.0, True)
    if scale is None:
        a.force[:4] = 2.0
        lj.run(m, counts, nbrs, a)
        assert np.all(a.force[:4] == 2.0)
        return
    lj.run(m, counts, nbrs, a)
    xf, yf = 0.22156665 * scale, 1.3825009 * scale
    exp = [[-xf, +yf, 0], [-xf, -yf, 0], [+xf, +yf, 0], [+xf, -yf, 0]]
    for got, e in zip(a.force[:4], exp):
        for gi, ei in zip(got, e):
            expect_float_eq(gi, ei)


def test_grid_fixture_multires_ghosts(orc):
    """test/GridFixture.hpp:27-78 with MultiResPeriodicGhostExchange
    (communication/MultiResPeriodicGhostExchange.test.cpp:39-54): every ghost
    molecule carries all of its atoms and ghost atoms map to real atoms."""
    sd = orc.subdomain([0, 0, 0], [3, 3, 3], 0.7)
    apm = 2
    mpos = np.array([(x + 0.5, y + 0.5, z + 0.5) for x in range(3) for y in range(3)
                     for z in range(3)])
    m = orc.Molecules(300)
    m.pos[:27] = mpos
    m.atomsOffset[:27] = np.arange(27) * apm
    m.numAtoms[:27] = apm
    m.numLocal = 27
    apos = np.repeat(mpos, apm, axis=0) + np.tile([[0, 0, 0], [0.1, 0.2, 0.3]], (27, 1))
    a = orc.Atoms.from_positions(apos, capacity=600)
    corr = orc.multires_create_ghosts(m, a, sd)
    assert m.numGhost == 98
    assert a.numGhost == 98 * apm
    g = np.arange(a.numLocal, a.n)
    assert np.all(corr[g] >= 0) and np.all(corr[g] < a.numLocal)
    d = a.pos[g] - a.pos[corr[g]]
    assert np.allclose(np.abs(d) % 3.0, 0)


def test_normal_generator_accuracy_and_moments(orc):
    """The Langevin normals: FP32 Box-Muller with our own ln and sin/cos on the
    23-bit uniforms of one Philox block; within 1e-6 of the exact Box-Muller of
    the same uniforms, and standard-normal moments."""
    import ctypes as C

    L = orc.lib()
    out = np.zeros(3)
    r = (C.c_uint32 * 4)()
    vals, worst = [], 0.0
    for a in range(20000):
        L.orc_philox4x32_10((C.c_uint32 * 4)(a, 0, 11, 0), (C.c_uint32 * 2)(5, 0), r)
        u = [((x >> 9) + 0.5) * 2.0 ** -23 for x in r]
        ra, rb = np.sqrt(-2 * np.log(u[0])), np.sqrt(-2 * np.log(u[2]))
        exact = [ra * np.cos(2 * np.pi * u[1]), ra * np.sin(2 * np.pi * u[1]), rb * np.cos(2 * np.pi * u[3])]
        L.orc_normal_from_counter(C.c_uint64(5), C.c_uint64(11), C.c_uint64(a),
                                  out.ctypes.data_as(C.POINTER(C.c_double)))
        worst = max(worst, float(np.max(np.abs(out - exact))))
        vals.append(out.copy())
    v = np.array(vals)
    assert worst < 1e-6
    assert np.all(np.abs(v.mean(axis=0)) < 0.03)
    assert np.all(np.abs(v.var(axis=0) - 1.0) < 0.03)
    assert np.all(np.abs((v ** 4).mean(axis=0) / v.var(axis=0) ** 2 - 3.0) < 0.15)


def test_analysis_kats(orc):
    """analysis/KineticEnergy.test.cpp:22-50 and SystemMomentum.test.cpp:23-42,
    and getPressure (analysis/Pressure.cpp:23-51) on a hand-computed case."""
    a = orc.Atoms(3)
    a.vel[:3] = [[2, 0, 0], [-0.0, -8, -0.0], [0, 0, 16]]
    a.mass[:3] = [1.0, 2.0, 0.5]
    a.numLocal = 3
    expect_float_eq(orc.kinetic_energy(a), (4 + 2 * 64 + 0.5 * 256) * 0.5)
    b = orc.Atoms(2)
    b.vel[:2] = [[2, 3, 4], [-4, -8, -16]]
    b.numLocal = 2
    for got, want in zip(orc.system_momentum(b), (-2, -5, -12)):
        expect_float_eq(got, want)
    # pressure: one local and one ghost atom, volume 2 * 3 * 4
    c = orc.Atoms(2)
    c.pos[:2] = [[1, 2, 3], [0.5, 0, 0]]
    c.vel[:2] = [[1, 0, 0], [0, 2, 0]]
    c.force[:2] = [[1, 1, 1], [4, 0, 0]]
    c.mass[:2] = [2.0, 1.0]
    c.numLocal, c.numGhost = 1, 1
    sd = orc.subdomain([0, 0, 0], [2, 3, 4], 0.5)
    assert orc.pressure(c, sd) == (2.0 + 6.0 + 4.0 + 2.0) / (3 * 24.0)
