"""GPU parity of the LJ hot path against the oracle, through the C ABI.

Bars: ghost sets, cell ids and neighbour pair sets are bit-exact; the
integrators and the ghost update / fold-back are bitwise equal (same FP64
operation order); FP64 forces agree to 1e-10 relative per atom (floored at
1e-4 of the RMS force), energy and virial to 1e-10 relative (only the
summation order differs); the mixed form stays within 1e-6 of the
FP64 forces normalised by the RMS force (the precision bound), with the
per-atom relative error reported.
"""
import numpy as np
import pytest

from conftest import FP64_RTOL, assert_fp64_forces, expect_float_eq, per_atom_rel_err

pytestmark = pytest.mark.gpu



@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


def espp_setup(M, orc, espp):
    g, pos = espp
    L, rc, skin = g["box"], g["rc"], g["skin"]
    sd_o = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    sd_g = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    return g, pos, L, rc, skin, sd_o, sd_g


def test_ghosts_bit_exact(M, orc, espp):
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ao = orc.Atoms.from_positions(pos, capacity=60000)
    corr_o = orc.create_ghosts(ao, sd_o)
    ag = M.Atoms.from_arrays(pos, capacity=40000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    assert ag.numGhostAtoms == g["num_ghost"] == ao.numGhost
    d = ag.download()
    np.testing.assert_array_equal(d["pos"], ao.pos[: ao.n])
    np.testing.assert_array_equal(gl.correspondingRealAtom(ao.n)[ao.numLocal:], corr_o[ao.numLocal: ao.n])


def test_cell_ids_bit_exact(M, orc, espp):
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ag = M.Atoms.from_arrays(pos)
    gmin, gmax = sd_o.minGhostCorner[:], sd_o.maxGhostCorner[:]
    cg = M.cell_index(ag, len(pos), gmin, gmax, rc + skin)
    nc, rdx = orc.cell_grid(gmin, gmax, rc + skin)
    co = orc.cell_index(pos, gmin, nc, rdx)
    np.testing.assert_array_equal(cg, co)


def test_half_list_pair_set_bit_exact(M, orc, espp):
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ao = orc.Atoms.from_positions(pos, capacity=60000)
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 64)
    ag = M.Atoms.from_arrays(pos, capacity=60000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 60)
    assert vl.total_pairs == g["num_pairs"]
    cg, ng = vl.download(64)
    np.testing.assert_array_equal(cg, co)
    # identical (i, j) sets per row, hence identical canonical pair sets
    for i in range(0, len(cg), 997):
        assert sorted(ng[i, : cg[i]]) == sorted(no[i, : co[i]])
    kg = orc.canonical_pairs(cg, ng, corr, ao.numLocal)
    ko = orc.canonical_pairs(co, no, corr, ao.numLocal)
    np.testing.assert_array_equal(kg, ko)


def test_list_capacity_grows(M, orc, espp):
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ag = M.Atoms.from_arrays(pos, capacity=60000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 4)
    assert vl.total_pairs == g["num_pairs"]
    assert vl.s.maxNeighbors > 4


def lj_forces_oracle(orc, ao, corr, co, no, tab, rc, pred_=None):
    ao.force[:] = 0
    E, W = orc.lj_apply(tab, rc * rc, ao, co, no, pred_)
    return E, W


def test_espp_energy_and_fp64_forces(M, orc, espp):
    """tests/LennardJones/LennardJones.cpp:124-128 on the GPU, plus per-atom parity."""
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ao = orc.Atoms.from_positions(pos, capacity=60000)
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 64)
    tab = orc.lj_table(0.0, rc, 1.0, 1.0, 1, False)
    Eo, Wo = lj_forces_oracle(orc, ao, corr, co, no, tab, rc)
    ag = M.Atoms.from_arrays(pos, capacity=60000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 60)
    lj = M.LennardJones(rc, 1.0, 1.0)
    ag.setForce(0.0)
    lj.apply(ag, vl)
    expect_float_eq(lj.getEnergy(), g["initial_energy"])
    assert abs(lj.getEnergy() - Eo) <= FP64_RTOL * abs(Eo)
    assert abs(lj.getVirial() - Wo) <= FP64_RTOL * abs(Wo)
    Fg = ag.getForce()
    assert_fp64_forces(Fg, ao.force[: ao.n], "ESPP before fold-back")
    # fold ghost forces back: gather order is the reference's serial order
    gl.contributeBackGhostToReal(ag)
    orc.ghost_to_real(ao, corr)
    Fg = ag.getForce()
    assert_fp64_forces(Fg[: ao.numLocal], ao.force[: ao.numLocal], "ESPP")
    assert np.all(Fg[ao.numLocal:] == 0)


def test_lj_table_bit_exact(M, orc):
    for cap, shifted in ((0.0, False), (0.7, True), (0.78420, True)):
        tg = M.LennardJones(2.5, 1.0, 1.0, cap, is_shifted=shifted).params()[0]
        to = orc.lj_table(cap, 2.5, 1.0, 1.0, 1, shifted)[0]
        for f in ("ff1", "ff2", "ef1", "ef2", "rcSqr", "cappingDistance", "cappingDistanceSqr", "shift"):
            assert getattr(tg, f) == getattr(to, f), f
        if cap > 0:
            assert tg.cappingCoeff == to.cappingCoeff
            assert tg.energyAtCappingPoint == to.energyAtCappingPoint


def random_fluid(n, L, seed, min_dist=0.85):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, L, (n, 3))
    return pts


@pytest.mark.parametrize("cap,shifted,pkind", [
    (0.0, True, None),
    (0.9, True, None),             # capped branch taken for close pairs
    (0.0, False, "either"),        # apply_if, examples/04 isInNoCapRegion form
    (0.7, True, "both"),           # apply_if, examples/04 isInCappingRegion form
])
def test_fp64_apply_if_random(M, orc, cap, shifted, pkind):
    L = 12.0
    pos = random_fluid(1200, L, 7)
    rc, skin = 2.5, 0.3
    sd_o = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    sd_g = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    ao = orc.Atoms.from_positions(pos, capacity=8000)
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 96)
    tab = orc.lj_table(cap, rc, 1.0, 1.0, 1, shifted)
    if pkind is None:
        po, pg = None, None
    else:
        kind = orc.PRED_EITHER_IN_SLAB if pkind == "either" else orc.PRED_BOTH_IN_SLAB
        lo, hi = (0.0, 3.0) if pkind == "either" else (3.0, 5.0)
        po = orc.pred(kind, 0, L / 2, lo, hi)
        pg = M.pred(kind, 0, L / 2, lo, hi)
    Eo, Wo = lj_forces_oracle(orc, ao, corr, co, no, tab, rc, po)
    ag = M.Atoms.from_arrays(pos, capacity=8000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 60)
    lj = M.LennardJones(rc, 1.0, 1.0, cap, is_shifted=shifted)
    ag.setForce(0.0)
    lj.apply_if(ag, vl, pg)
    Fg = ag.getForce()
    assert_fp64_forces(Fg, ao.force[: ao.n])
    assert abs(lj.getEnergy() - Eo) <= FP64_RTOL * max(abs(Eo), 1.0)
    assert abs(lj.getVirial() - Wo) <= FP64_RTOL * max(abs(Wo), 1.0)


@pytest.mark.parametrize("num_types_index", [1, 3])
def test_fp64_multi_type_random(M, orc, num_types_index):
    """Three atom types with per-pair parameters.  num_types_index 1 is the
    reference's type index (LennardJones.cpp:52 sets numTypes_ to 1, so the
    pair (i, j) reads entry type_i + type_j); 3 is the full table."""
    L, rc, skin = 12.0, 2.5, 0.3
    pos = random_fluid(1500, L, 21)
    rng = np.random.default_rng(21)
    types = rng.integers(0, 3, len(pos))
    sig = np.array([[1.0, 1.1, 0.9], [1.1, 1.2, 1.0], [0.9, 1.0, 0.8]]).ravel()
    eps = np.array([[1.0, 0.7, 1.3], [0.7, 0.5, 0.9], [1.3, 0.9, 1.6]]).ravel()
    cap = np.full(9, 0.8)
    rcs = np.full(9, rc)
    sd_o = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    sd_g = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    ao = orc.Atoms.from_positions(pos, capacity=9000)
    ao.type[: len(pos)] = types
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 96)
    tab = orc.lj_table(cap, rcs, sig, eps, 3, True)
    ao.force[:] = 0
    Eo, Wo = orc.lj_apply(tab, rc * rc, ao, co, no, None, num_types_index)
    ag = M.Atoms.from_arrays(pos, capacity=9000, type=types)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 60)
    lj = M.LennardJones(rcs, sig, eps, cap, num_types=3, is_shifted=True, num_types_index=num_types_index)
    for k, p in enumerate(lj.params()):
        assert (p.ff1, p.ff2, p.shift) == (tab[k].ff1, tab[k].ff2, tab[k].shift)
    ag.setForce(0.0)
    lj.apply(ag, vl)
    Fg = ag.getForce()
    assert_fp64_forces(Fg, ao.force[: ao.n])
    assert abs(lj.getEnergy() - Eo) <= FP64_RTOL * max(abs(Eo), 1.0)
    assert abs(lj.getVirial() - Wo) <= FP64_RTOL * max(abs(Wo), 1.0)
    with pytest.raises(M.MrmdError):
        lj.apply(ag, vl, precision=M.PREC_MIXED)


def test_mixed_precision_force_error(M, orc, espp):
    """Mixed form on the ESPP system: max |dF| / rms|F| <= 1e-6."""
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ao = orc.Atoms.from_positions(pos, capacity=60000)
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 64)
    tab = orc.lj_table(0.0, rc, 1.0, 1.0, 1, True)
    Eo, Wo = lj_forces_oracle(orc, ao, corr, co, no, tab, rc)
    orc.ghost_to_real(ao, corr)
    ag = M.Atoms.from_arrays(pos, capacity=60000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 60)
    lj = M.LennardJones(rc, 1.0, 1.0, is_shifted=True)
    ag.setForce(0.0)
    lj.apply(ag, vl, precision=M.PREC_MIXED)
    gl.contributeBackGhostToReal(ag)
    Fg = ag.getForce()[: ao.numLocal]
    Fo = ao.force[: ao.numLocal]
    d = np.linalg.norm(Fg - Fo, axis=1)
    rms = np.sqrt((np.linalg.norm(Fo, axis=1) ** 2).mean())
    assert d.max() / rms <= 1e-6, d.max() / rms
    assert abs(lj.getEnergy() - Eo) <= 1e-7 * abs(Eo)
    assert abs(lj.getVirial() - Wo) <= 1e-7 * abs(Wo)


def test_list_rows_offset_by_begin(M, orc):
    """A list built over particles [begin, end) with begin > 0: its row r is
    particle begin + r, as in the reference, which indexes Cabana's list by
    absolute particle (LennardJones.hpp:146-170; the rows outside
    [begin, end) are empty).  FP64 per atom against the oracle run on the
    same list in absolute form, and the mixed form within its bar."""
    L, rc, skin = 12.0, 2.5, 0.3
    pos = random_fluid(1200, L, 31)
    b, e = 300, 900
    sd_o = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    sd_g = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    ao = orc.Atoms.from_positions(pos, capacity=8000)
    corr = orc.create_ghosts(ao, sd_o)
    co, no = orc.build_half_list(ao.pos, ao.n, b, e, rc + skin, sd_o.minGhostCorner,
                                 sd_o.maxGhostCorner, 1.0, 96)
    ca = np.zeros(ao.numLocal, np.int32)
    na = np.zeros((ao.numLocal, no.shape[1]), np.int32)
    ca[b:e], na[b:e] = co, no
    tab = orc.lj_table(0.0, rc, 1.0, 1.0, 1, True)
    Eo, Wo = lj_forces_oracle(orc, ao, corr, ca, na, tab, rc)
    ag = M.Atoms.from_arrays(pos, capacity=8000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    vl = M.HalfVerletList()
    vl.build(ag, b, e, rc + skin, 1.0, sd_g.minGhostCorner, sd_g.maxGhostCorner, 60)
    assert vl.total_pairs == int(co.sum())
    lj = M.LennardJones(rc, 1.0, 1.0, is_shifted=True)
    ag.setForce(0.0)
    lj.apply(ag, vl)
    Fg = ag.getForce()
    assert_fp64_forces(Fg, ao.force[: ao.n], "begin > 0")
    assert np.all(Fg[:b][np.all(ao.force[:b] == 0, axis=1)] == 0)
    assert abs(lj.getEnergy() - Eo) <= FP64_RTOL * abs(Eo)
    assert abs(lj.getVirial() - Wo) <= FP64_RTOL * abs(Wo)
    ag.setForce(0.0)
    lj.apply(ag, vl, precision=M.PREC_MIXED)
    Fm = ag.getForce()
    rms = np.sqrt((np.linalg.norm(ao.force[: ao.n], axis=1) ** 2).mean())
    assert np.linalg.norm(Fm - ao.force[: ao.n], axis=1).max() / rms <= 1e-6
    assert abs(lj.getEnergy() - Eo) <= 1e-7 * abs(Eo)


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_position_reported_at_list_build(M, bad):
    """A NaN or infinite coordinate, written into the host array before the
    upload, makes the next list build return MRMD_ERR_NONFINITE (the
    reference asserts on NaN forces, LJ_IdealGas.cpp:140-155); the context
    stays usable."""
    L, rc, skin = 12.0, 2.5, 0.3
    pos = random_fluid(1200, L, 41)
    pos[517, 1] = bad
    sd = M.Subdomain([0, 0, 0], [L] * 3, rc + skin)
    ag = M.Atoms.from_arrays(pos, capacity=8000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd)
    vl = M.HalfVerletList()
    with pytest.raises(M.MrmdError) as ei:
        vl.build(ag, 0, ag.numLocalAtoms, rc + skin, 1.0, sd.minGhostCorner, sd.maxGhostCorner, 60)
    assert ei.value.code == -4
    # the same context builds a clean list afterwards
    ok = random_fluid(1200, L, 41)
    a2 = M.Atoms.from_arrays(ok, capacity=8000)
    g2 = M.GhostLayer()
    g2.createGhostAtoms(a2, sd)
    v2 = M.HalfVerletList()
    v2.build(a2, 0, a2.numLocalAtoms, rc + skin, 1.0, sd.minGhostCorner, sd.maxGhostCorner, 60)
    assert v2.total_pairs > 0


def test_integrators_bitwise(M, orc, espp):
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    rng = np.random.default_rng(3)
    n = len(pos)
    vel = rng.normal(0, 1, (n, 3))
    force = rng.normal(0, 50, (n, 3))
    mass = rng.uniform(0.5, 2.0, n)
    ao = orc.Atoms.from_positions(pos)
    ao.vel[:n], ao.force[:n], ao.mass[:n] = vel, force, mass
    ag = M.Atoms.from_arrays(pos, vel=vel, force=force, mass=mass)
    mo = orc.vv_pre(ao, 0.005)
    mg = M.VelocityVerlet.preForceIntegrate(ag, 0.005)
    d = ag.download(n)
    np.testing.assert_array_equal(d["pos"], ao.pos[:n])
    np.testing.assert_array_equal(d["vel"], ao.vel[:n])
    assert mo == mg
    orc.vv_post(ao, 0.005)
    M.VelocityVerlet.postForceIntegrate(ag, 0.005)
    np.testing.assert_array_equal(ag.getVel(n), ao.vel[:n])


def test_vv_single_atom_kat(M):
    """action/VelocityVerlet.test.cpp:27-71"""
    a = M.Atoms.from_arrays([[2, 3, 4]], vel=[[7, 5, 3]], force=[[9, 7, 8]], mass=1.5)
    M.VelocityVerlet.preForceIntegrate(a, 4.0)
    d = a.download(1)
    for got, exp in zip(d["vel"][0], (19, 14.333333, 13.666667)):
        expect_float_eq(got, exp)
    for got, exp in zip(d["pos"][0], (78, 60.333332, 58.666668)):
        expect_float_eq(got, exp)


def test_ghost_update_and_map_bitwise(M, orc, espp):
    g, pos, L, rc, skin, sd_o, sd_g = espp_setup(M, orc, espp)
    ao = orc.Atoms.from_positions(pos, capacity=60000)
    corr = orc.create_ghosts(ao, sd_o)
    ag = M.Atoms.from_arrays(pos, capacity=60000)
    gl = M.GhostLayer()
    gl.createGhostAtoms(ag, sd_g)
    rng = np.random.default_rng(5)
    shift = rng.normal(0, 0.05, (ao.numLocal, 3))
    newpos = pos + shift
    ao.pos[: ao.numLocal] = newpos
    ag.upload(ao.numLocal, ao.numGhost, pos=ao.pos[: ao.n])
    orc.update_ghosts(ao, corr, sd_o)
    gl.updateGhostAtoms(ag, sd_g)
    np.testing.assert_array_equal(ag.getPos(), ao.pos[: ao.n])
    # periodic wrap of real atoms
    ao2 = orc.Atoms.from_positions(newpos)
    orc.map_into_domain(ao2, sd_o)
    ag2 = M.Atoms.from_arrays(newpos)
    gl.exchangeRealAtoms(ag2, sd_g)
    np.testing.assert_array_equal(ag2.getPos(), ao2.pos[: ao2.numLocal])


def test_ghost_exchange_grid27(M):
    """communication/GhostExchange.test.cpp:119-153 on the GPU."""
    pts = np.array([(x + 0.5, y + 0.5, z + 0.5) for x in range(3) for y in range(3) for z in range(3)])
    a = M.Atoms.from_arrays(pts, capacity=200)
    gl = M.GhostLayer()
    gl.createGhostAtoms(a, M.Subdomain([0, 0, 0], [3, 3, 3], 0.7))
    assert a.numGhostAtoms == 98
    corr = gl.correspondingRealAtom(a.size)
    assert np.all(corr[:27] == -1) and np.all((corr[27:] >= 0) & (corr[27:] < 27))


def test_empty_and_tiny_inputs(M):
    a = M.Atoms(4)
    sd = M.Subdomain([0, 0, 0], [10, 10, 10], 2.8)
    gl = M.GhostLayer()
    gl.createGhostAtoms(a, sd)
    assert a.numGhostAtoms == 0
    vl = M.HalfVerletList()
    vl.build(a, 0, 0, 2.8, 1.0, sd.minGhostCorner, sd.maxGhostCorner, 8, n_pos=0)
    lj = M.LennardJones(2.5, 1.0, 1.0)
    lj.apply(a, vl)
    assert lj.getEnergy() == 0.0
    assert M.VelocityVerlet.preForceIntegrate(a, 0.005) == 0.0
    # one pair
    b = M.Atoms.from_arrays([[5.0, 5.0, 5.0], [6.1, 5.0, 5.0]])
    vl.build(b, 0, 2, 2.8, 1.0, sd.minGhostCorner, sd.maxGhostCorner, 8)
    assert vl.total_pairs == 1
    b.setForce(0.0)
    lj.apply(b, vl)
    f = b.getForce()
    np.testing.assert_allclose(f[0], -f[1], rtol=0, atol=1e-15)


def test_bad_arguments_raise(M):
    a = M.Atoms(4)
    vl = M.HalfVerletList()
    with pytest.raises(M.MrmdError):
        vl.build(a, 0, 10, 2.8, 1.0, [0, 0, 0], [1, 1, 1], 8, n_pos=4)
    with pytest.raises(M.MrmdError):
        M.LennardJones(2.5, 1.0, 1.0).apply_if(a, vl, M.pred(kind=99))
