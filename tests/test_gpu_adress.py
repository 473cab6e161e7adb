"""GPU parity of the AdResS pieces (Slab / UpdateMolecules, ContributeMoleculeForceToAtoms,
LJ_IdealGas, MultiResGhostLayer), the thermodynamic force and the Langevin
integrator against the oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import assert_fp64_forces, expect_float_eq

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


def single_site_system(n, box, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 1, (n, 3)) * np.asarray(box)
    return pos


def upload_molecules(M, mo, n_local, n_ghost=0):
    m = M.Molecules(max(mo.capacity, 4))
    n = n_local + n_ghost
    m.upload(n_local, n_ghost, pos=mo.pos[:n], force=mo.force[:n], lambda_=mo.lambda_[:n],
             modulated_lambda=mo.modulatedLambda[:n], grad_lambda=mo.gradLambda[:n],
             atoms_offset=mo.atomsOffset[:n], num_atoms=mo.numAtoms[:n])
    return m


def test_slab_update_molecules(M, orc):
    rng = np.random.default_rng(1)
    n = 5000
    apos = rng.uniform(0, 120, (2 * n, 3))
    rel = np.full(2 * n, 0.5)
    mo = orc.Molecules(n)
    mo.atomsOffset[:n] = np.arange(n) * 2
    mo.numAtoms[:n] = 2
    mo.numLocal = n
    ao = orc.Atoms.from_positions(apos)
    ao.relativeMass[: 2 * n] = rel
    for nu, itype in ((1, 0), (2, 0), (1, 1)):
        so = orc.slab([60, 12, 12], 30.0, 10.0, nu, itype)
        orc.update_molecules(mo, ao, so)
        m = upload_molecules(M, mo, n)
        a = M.Atoms.from_arrays(apos, relative_mass=rel)
        M.UpdateMolecules.update(m, a, M.Slab([60, 12, 12], 30.0, 10.0, nu, itype))
        d = m.download(n)
        np.testing.assert_array_equal(d["pos"], mo.pos[:n])
        np.testing.assert_allclose(d["lambda_"], mo.lambda_[:n], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(d["modulatedLambda"], mo.modulatedLambda[:n], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(d["gradLambda"], mo.gradLambda[:n], rtol=1e-12, atol=1e-15)


def test_contribute_molecule_force(M, orc):
    """action/ContributeMoleculeForceToAtoms.test.cpp:27-51 + random bitwise parity"""
    m = M.Molecules(2)
    m.upload(2, 0, pos=np.zeros((2, 3)), force=[[5, 6, 7], [0, 0, 0]], lambda_=np.zeros(2),
             modulated_lambda=np.zeros(2), grad_lambda=np.zeros((2, 3)), atoms_offset=[0, 2],
             num_atoms=[2, 2])
    a = M.Atoms.from_arrays([[1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0]], mass=[1, 3, 1, 3],
                            relative_mass=[0.25, 0.75, 0.25, 0.75])
    M.ContributeMoleculeForceToAtoms.update(m, a)
    f = a.getForce(4)
    for got, exp in zip(f[0], np.array([5, 6, 7]) * 0.25):
        expect_float_eq(got, exp)
    for got, exp in zip(f[1], np.array([5, 6, 7]) * 0.75):
        expect_float_eq(got, exp)


@pytest.mark.parametrize("lam,scale", [(0.0, None), (0.5, 0.5), (1.0, 1.0)])
def test_lj_ideal_gas_kat(M, lam, scale):
    """action/LJ_IdealGas.test.cpp:140-220 (CG / HY / AT)"""
    m = M.Molecules(2)
    m.upload(2, 0, pos=[[-0.5, 0, 0], [0.5, 0, 0]], force=np.zeros((2, 3)), lambda_=np.zeros(2),
             modulated_lambda=[lam, lam], grad_lambda=np.zeros((2, 3)), atoms_offset=[0, 2],
             num_atoms=[2, 2])
    a = M.Atoms.from_arrays([[-0.5, -0.5, 0], [-0.5, 0.5, 0], [0.5, -0.5, 0], [0.5, 0.5, 0]],
                            relative_mass=0.5)
    vl = M.HalfVerletList()
    vl.build(m, 0, 2, 2.0, 1.0, [-1, -1, -1], [1, 1, 1], 4)
    sigma = 0.9
    lj = M.LJ_IdealGas(0.0, 2.5 * sigma, sigma, 2.0, True)
    if scale is None:
        a.setForce(2.0)
        lj.run(m, vl, a)
        assert np.all(a.getForce(4) == 2.0)
        return
    a.setForce(0.0)
    lj.run(m, vl, a)
    f = a.getForce(4)
    xf, yf = 0.22156665 * scale, 1.3825009 * scale
    exp = [[-xf, +yf, 0], [-xf, -yf, 0], [+xf, +yf, 0], [+xf, -yf, 0]]
    for got, e in zip(f, exp):
        for gi, ei in zip(got, e):
            expect_float_eq(gi, ei)


def adress_system(orc, n=3000, box=(40.0, 12.0, 12.0), seed=4, apm=1):
    rc, skin = 2.5, 0.3
    rng = np.random.default_rng(seed)
    mpos = rng.uniform(0, 1, (n, 3)) * np.asarray(box)
    offs = rng.normal(0, 0.15, (n * apm, 3)) if apm > 1 else np.zeros((n, 3))
    apos = np.repeat(mpos, apm, axis=0) + offs
    sd = orc.subdomain([0, 0, 0], list(box), rc + skin)
    mo = orc.Molecules(n * 8)
    mo.pos[:n] = mpos
    mo.atomsOffset[:n] = np.arange(n) * apm
    mo.numAtoms[:n] = apm
    mo.numLocal = n
    ao = orc.Atoms.from_positions(apos, capacity=n * apm * 8)
    ao.relativeMass[: n * apm] = 1.0 / apm
    slab = orc.slab([box[0] / 2, box[1] / 2, box[2] / 2], 10.0, 5.0, 1)
    orc.update_molecules(mo, ao, slab)
    orc.multires_map_into_domain(sd, mo, ao)
    corr = orc.multires_create_ghosts(mo, ao, sd)
    orc.update_molecules(mo, ao, slab)
    return mo, ao, corr, sd, slab, (rc, skin, box)


def test_multires_ghosts_bit_exact(M, orc):
    for apm in (1, 3):
        mo, ao, corr, sd, slab, (rc, skin, box) = adress_system(orc, n=1500, apm=apm)
        n = mo.numLocal
        # rebuild on the GPU from the local part
        m = M.Molecules(n)
        m.upload(n, 0, pos=mo.pos[:n], force=np.zeros((n, 3)), lambda_=mo.lambda_[:n],
                 modulated_lambda=mo.modulatedLambda[:n], grad_lambda=mo.gradLambda[:n],
                 atoms_offset=mo.atomsOffset[:n], num_atoms=mo.numAtoms[:n])
        a = M.Atoms.from_arrays(ao.pos[: ao.numLocal], relative_mass=1.0 / apm)
        gl = M.MultiResGhostLayer()
        sdg = M.Subdomain([0, 0, 0], list(box), rc + skin)
        gl.createGhostAtoms(m, a, sdg)
        assert m.numGhostMolecules == mo.numGhost and a.numGhostAtoms == ao.numGhost
        # the oracle fixture recomputes every centre of mass after ghost creation
        M.UpdateMolecules.update(m, a, M.Slab([box[0] / 2, box[1] / 2, box[2] / 2], 10.0, 5.0, 1))
        d = m.download()
        np.testing.assert_array_equal(d["pos"], mo.pos[: mo.numLocal + mo.numGhost])
        np.testing.assert_array_equal(d["atomsOffset"], mo.atomsOffset[: mo.numLocal + mo.numGhost])
        np.testing.assert_array_equal(a.getPos(), ao.pos[: ao.n])
        np.testing.assert_array_equal(gl.correspondingRealAtom(ao.n)[ao.numLocal:], corr[ao.numLocal: ao.n])


@pytest.mark.parametrize("apm", [1, 2])
def test_lj_ideal_gas_random_vs_oracle(M, orc, apm):
    mo, ao, corr, sd, slab, (rc, skin, box) = adress_system(orc, n=2500, apm=apm)
    nm = mo.numLocal + mo.numGhost
    co, no = orc.build_half_list(mo.pos, nm, 0, mo.numLocal, rc + skin, sd.minGhostCorner,
                                 sd.maxGhostCorner, 1.0, 96)
    m = upload_molecules(M, mo, mo.numLocal, mo.numGhost)
    a = M.Atoms.from_arrays(ao.pos[: ao.n], relative_mass=ao.relativeMass[: ao.n],
                            capacity=ao.capacity)
    a.numLocalAtoms, a.numGhostAtoms = ao.numLocal, ao.numGhost
    vl = M.HalfVerletList()
    vl.build(m, 0, mo.numLocal, rc + skin, 1.0, sd.minGhostCorner[:], sd.maxGhostCorner[:], 64)
    cg, ng = vl.download(96)
    np.testing.assert_array_equal(cg, co)
    ljo = orc.LJIdealGas(0.0, rc, 1.0, 1.0, True)
    ljg = M.LJ_IdealGas(0.0, rc, 1.0, 1.0, True)
    for run in range(3):  # run 0 samples and updates the running mean; runs 1, 2 do not sample
        ao.force[:] = 0
        mo.force[:] = 0
        a.setForce(0.0)
        m.setForce(0.0)
        Eo = ljo.run(mo, co, no, ao)
        Eg = ljg.run(m, vl, a)
        assert_fp64_forces(a.getForce(), ao.force[: ao.n], "LJ_IdealGas atoms")
        dm = m.download()
        assert_fp64_forces(dm["force"], mo.force[:nm], "LJ_IdealGas molecules")
        assert abs(Eg - Eo) <= 1e-10 * max(abs(Eo), 1.0)
    comp = ljg.compensation()
    np.testing.assert_allclose(comp["mean"], ljo.mean, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(comp["counter"], ljo.counter, rtol=0, atol=0)
    assert comp["runCounter"] == 3


def test_lj_ideal_gas_mixed_precision(M, orc):
    mo, ao, corr, sd, slab, (rc, skin, box) = adress_system(orc, n=2500)
    nm = mo.numLocal + mo.numGhost
    co, no = orc.build_half_list(mo.pos, nm, 0, mo.numLocal, rc + skin, sd.minGhostCorner,
                                 sd.maxGhostCorner, 1.0, 96)
    m = upload_molecules(M, mo, mo.numLocal, mo.numGhost)
    a = M.Atoms.from_arrays(ao.pos[: ao.n], capacity=ao.capacity)
    a.numLocalAtoms, a.numGhostAtoms = ao.numLocal, ao.numGhost
    vl = M.HalfVerletList()
    vl.build(m, 0, mo.numLocal, rc + skin, 1.0, sd.minGhostCorner[:], sd.maxGhostCorner[:], 64)
    ljo = orc.LJIdealGas(0.0, rc, 1.0, 1.0, True)
    ljg = M.LJ_IdealGas(0.0, rc, 1.0, 1.0, True)
    ao.force[:] = 0
    a.setForce(0.0)
    ljo.run(mo, co, no, ao)
    ljg.run(m, vl, a, precision=M.PREC_MIXED)
    Fo = ao.force[: ao.n]
    rms = np.sqrt((np.linalg.norm(Fo, axis=1) ** 2).mean())
    err = np.linalg.norm(a.getForce() - Fo, axis=1).max() / rms
    assert err <= 1e-6, err


def tf_fixture(M, orc):
    """action/ThermodynamicForce.test.cpp:79-94"""
    sdo = orc.subdomain([0, 0, 0], [10, 1, 1], 1.0)
    sdg = M.Subdomain([0, 0, 0], [10, 1, 1], 1.0)
    tfo = orc.ThermodynamicForce([1.0], sdo, 1.0, [1.0])
    tfg = M.ThermodynamicForce([1.0], sdg, 1.0, [1.0])
    tfo.force[:, 0] = np.arange(10)
    tfg.setForce(np.arange(10.0).reshape(10, 1))
    return tfo, tfg


def test_tf_kats_on_gpu(M, orc):
    """action/ThermodynamicForce.test.cpp:108-245"""
    x = np.arange(100) / 10.0
    uni = np.stack([x, 0 * x, 0 * x], 1)
    xs = [i + 0.5 for i in range(10) for _ in range(i)]
    non = np.stack([xs, np.zeros(45), np.zeros(45)], 1)
    tfo, tfg = tf_fixture(M, orc)
    tfg.sample(M.Atoms.from_arrays(uni))
    assert np.all(tfg.getDensityProfile()[:, 0] == 10)
    a = M.Atoms.from_arrays(uni)
    tfg.apply(a)
    np.testing.assert_array_equal(a.getForce(100)[:, 0], np.floor(x))
    a = M.Atoms.from_arrays(uni)
    tfg.applyInterpolated_if(a, M.pred(M.PRED_IN_OPEN_INTERVAL, 0, 0, 0.5, 4.5))
    f = a.getForce(100)[:, 0]
    sel = (x > 0.5) & (x < 4.5)
    for xi, fi, s in zip(x, f, sel):
        if s:
            expect_float_eq(fi, xi - 0.5)
        else:
            assert fi == 0
    tfo, tfg = tf_fixture(M, orc)
    tfg.sample(M.Atoms.from_arrays(non))
    tfg.update(1.0, 0.0)
    for i, v in enumerate(tfg.getForce()[:, 0]):
        expect_float_eq(v, i - 1.0)
    assert tfg.getNumberOfDensityProfileSamples() == 0


def test_tf_random_vs_oracle(M, orc):
    rng = np.random.default_rng(9)
    box = [120.0, 24.0, 24.0]
    n = 30000
    sdo = orc.subdomain([0, 0, 0], box, 2.8)
    sdg = M.Subdomain([0, 0, 0], box, 2.8)
    for sym, per in ((False, False), (True, True)):
        tfo = orc.ThermodynamicForce([0.5], sdo, 1.2, [2.0], sym, per)
        tfg = M.ThermodynamicForce([0.5], sdg, 1.2, [2.0], sym, per)
        assert tfg.num_bins == tfo.force.shape[0] == 100
        for k in range(3):
            pos = rng.uniform(0, 1, (n, 3)) * box
            ao = orc.Atoms.from_positions(pos)
            tfo.sample(ao)
            tfg.sample(M.Atoms.from_arrays(pos))
        np.testing.assert_array_equal(tfg.getDensityProfile(), tfo.density)
        p1o = orc.pred(orc.PRED_IN_SLAB, 0, 60.0, 15.0, 25.0)
        p1g = M.pred(M.PRED_IN_SLAB, 0, 60.0, 15.0, 25.0)
        tfo.update(1.0, 3.0, p1o)
        tfg.update_if(1.0, 3.0, p1g)
        np.testing.assert_allclose(tfg.getForce(), tfo.force, rtol=1e-12, atol=1e-14)
        pos = rng.uniform(0, 1, (n, 3)) * box
        ao = orc.Atoms.from_positions(pos)
        a = M.Atoms.from_arrays(pos)
        tfo.apply(ao)
        tfg.apply(a)
        np.testing.assert_allclose(a.getForce(n), ao.force[:n], rtol=1e-12, atol=1e-14)
        ao.force[:] = 0
        a.setForce(0.0)
        tfo.apply_interpolated(ao)
        tfg.applyInterpolated_if(a)
        np.testing.assert_allclose(a.getForce(n), ao.force[:n], rtol=1e-12, atol=1e-14)
        lo, ro = tfo.mu()
        lg, rg = tfg.getMu()
        np.testing.assert_allclose([lg, rg], [lo, ro], rtol=1e-12, atol=1e-14)


def test_langevin_vs_oracle(M, orc):
    rng = np.random.default_rng(2)
    n = 20000
    pos = rng.uniform(0, 30, (n, 3))
    vel = rng.normal(0, 1, (n, 3))
    force = rng.normal(0, 5, (n, 3))
    for p in (None, "slab"):
        ao = orc.Atoms.from_positions(pos)
        ao.vel[:n], ao.force[:n] = vel, force
        a = M.Atoms.from_arrays(pos, vel=vel, force=force)
        po = None if p is None else orc.pred(orc.PRED_IN_SLAB, 0, 15.0, 5.0, 10.0)
        pg = None if p is None else M.pred(M.PRED_IN_SLAB, 0, 15.0, 5.0, 10.0)
        th = M.VelocityVerletLangevinThermostat(1.0, 1.0, seed=1234)
        mo = orc.langevin_pre(ao, 0.005, 1.0, 1.0, 1234, 7, po)
        mg = th.preForceIntegrate_apply_if(a, 0.005, pg, step=7)
        d = a.download(n)
        np.testing.assert_allclose(d["vel"], ao.vel[:n], rtol=1e-13, atol=1e-14)
        np.testing.assert_allclose(d["pos"], ao.pos[:n], rtol=1e-14, atol=1e-14)
        assert abs(mg - mo) <= 1e-12 * mo
