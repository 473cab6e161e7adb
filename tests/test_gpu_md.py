"""The fused LJ NVE stepper (examples/02 loop) against an oracle-driven loop."""
import numpy as np
import pytest

from conftest import per_atom_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


def fcc(cells, rho=0.8442):
    a = (4.0 / rho) ** (1.0 / 3.0)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(cells)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = ((g[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25) * a
    return pos, a * cells


def mb_velocities(n, T, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(0, np.sqrt(T), (n, 3))
    v -= v.mean(0)
    return v


def oracle_run(orc, pos, vel, L, nsteps, rc=2.5, skin=0.3, dt=0.005, K=10, observe=False):
    """examples/02_LennardJones_NVE.cpp:135-216 with a fixed rebuild interval.
    observe: each energy row also holds getKineticEnergy and getSystemMomentum
    after the step."""
    sd = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    a = orc.Atoms.from_positions(pos, capacity=len(pos) * 4)
    a.vel[: len(pos)] = vel
    tab = orc.lj_table(0.0, rc, 1.0, 1.0, 1, True)
    # initial forces
    corr = orc.create_ghosts(a, sd)
    co, no = orc.build_half_list(a.pos, a.n, 0, a.numLocal, rc + skin, sd.minGhostCorner,
                                 sd.maxGhostCorner, 1.0, 96)
    a.force[:] = 0
    orc.lj_apply(tab, rc * rc, a, co, no)
    orc.ghost_to_real(a, corr)
    energies = []
    for step in range(nsteps):
        orc.vv_pre(a, dt)
        if step % K == 0:
            a.numGhost = 0
            orc.map_into_domain(a, sd)
            corr = orc.create_ghosts(a, sd)
            co, no = orc.build_half_list(a.pos, a.n, 0, a.numLocal, rc + skin, sd.minGhostCorner,
                                         sd.maxGhostCorner, 1.0, 96)
        else:
            orc.update_ghosts(a, corr, sd)
        a.force[:] = 0
        E, W = orc.lj_apply(tab, rc * rc, a, co, no)
        orc.ghost_to_real(a, corr)
        orc.vv_post(a, dt)
        if observe:
            energies.append((E, W, orc.kinetic_energy(a), *orc.system_momentum(a)))
        else:
            energies.append((E, W))
    n = len(pos)
    return a.pos[:n].copy(), a.vel[:n].copy(), a.force[:n].copy(), np.array(energies)


def periodic_diff(a, b, L):
    d = a - b
    return d - L * np.round(d / L)


@pytest.mark.parametrize("graph,sort", [(False, False), (True, True)])
def test_fp64_trajectory_matches_oracle(M, orc, graph, sort):
    pos, L = fcc(6)  # 864 atoms
    rng = np.random.default_rng(11)
    pos = pos + rng.normal(0, 0.02, pos.shape)
    vel = mb_velocities(len(pos), 0.728, 1)
    steps = 25
    po, vo, fo, eo = oracle_run(orc, pos, vel, L, steps)
    sysm = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64, use_graph=graph,
                      sort_atoms=sort)
    eg = sysm.run(steps)
    pg, vg, fg = sysm.state()
    assert np.abs(periodic_diff(pg, po, L)).max() < 1e-11
    assert np.abs(vg - vo).max() < 1e-9
    np.testing.assert_allclose(eg[:, 0], eo[:, 0], rtol=1e-10)
    np.testing.assert_allclose(eg[:, 1], eo[:, 1], rtol=1e-10)
    st = sysm.stats()
    assert st["steps"] == steps and st["rebuilds"] >= 3


def test_mixed_stepper_is_deterministic_and_graph_invariant(M):
    pos, L = fcc(6)
    vel = mb_velocities(len(pos), 0.728, 2)
    runs = []
    for graph in (False, True, True):
        s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED, use_graph=graph)
        e = s.run(30)
        p, v, f = s.state()
        runs.append((e, p, v, f))
    for e, p, v, f in runs[1:]:
        # forces are written by their owning thread: positions and velocities
        # are bitwise reproducible; the energy is a sum of per-block partials
        # combined with atomics, reproducible to rounding
        np.testing.assert_array_equal(p, runs[0][1])
        np.testing.assert_array_equal(v, runs[0][2])
        np.testing.assert_allclose(e, runs[0][0], rtol=1e-13)


def test_mixed_cutoff_decision_at_scale(M):
    """256,000 atoms (~20M list pairs): the mixed form must place pairs at the
    cutoff exactly as FP64 does (the shifted LJ force jumps at rc)."""
    pos, L = fcc(40)
    rng = np.random.default_rng(7)
    pos = pos + rng.normal(0, 0.1, pos.shape)
    vel = mb_velocities(len(pos), 0.728, 4)
    ref = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64)
    mix = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED)
    ref.eval_forces()
    mix.eval_forces()
    fr = ref.state()[2]
    fm = mix.state()[2]
    rms = np.sqrt((np.linalg.norm(fr, axis=1) ** 2).mean())
    err = np.linalg.norm(fm - fr, axis=1).max() / rms
    assert err < 1e-6, err
    # per atom, floored at 0.1 of the RMS force (close contacts of the
    # jittered lattice give forces of thousands here)
    assert per_atom_rel_err(fm, fr, 0.1) < 1e-6
    assert mix.stats()["pairs"] > 1.9 * ref.stats()["pairs"]


def test_mixed_vs_fp64_forces(M):
    pos, L = fcc(8)  # 2048 atoms
    vel = mb_velocities(len(pos), 0.728, 3)
    ref = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64)
    mix = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED)
    # equilibrate in FP64, then compare forces on the same positions
    ref.run(200)
    p, v, f = ref.state()
    mix.set_state(p, v)
    ref.set_state(p, v)
    mix.run(1)
    ref.run(1)
    pm, vm, fm = mix.state()
    pr, vr, fr = ref.state()
    rms = np.sqrt((np.linalg.norm(fr, axis=1) ** 2).mean())
    err = np.linalg.norm(fm - fr, axis=1).max() / rms
    assert err < 1e-6, err
    assert per_atom_rel_err(fm, fr, 0.1) < 1e-6


def test_nve_drift_both_forms(M):
    """NVE energy drift of both forms: the slope of a least-squares line
    through (E_pot + E_kin) / N of every step, from the device-summed per-step
    energies, in epsilon per atom per 1000 tau.  Protocol of the benchmark's
    drift figure at a fifth of its length: 32,000 atoms (fcc 20^3, rho
    0.8442), 2,000 FP64 steps from the lattice at T 0.728, then 40,000 steps
    (200 tau) of each form from that state, for velocity seeds 7, 8 and 9.
    The energy of this protocol is a random walk (kicks from the force jump at
    rc), so a slope fitted over 200 tau scatters by ~1.5e-4 between seeds
    (sd of the mean of three ~0.9e-4); the means measured on a GB300 are
    ~1e-4 for both forms.  Limits: |mean| <= 5e-4 for each form, and the
    mixed mean within 5e-4 of the FP64 mean."""
    import bench

    ctx = M.default_context()
    r = bench.nve_drift(M, ctx, ["fp64", "mixed"], cells=20, equil=2000, steps=40000, seeds=(7, 8, 9))
    d64, dmx = r["fp64"]["drift"], r["mixed"]["drift"]
    assert abs(d64) <= 5e-4 and abs(dmx) <= 5e-4, r
    assert abs(dmx - d64) <= 5e-4, r


@pytest.mark.parametrize("split_radius,bound", [(0.0, 1e-6), (1.8, 5e-7), (2.8, 5e-8)])
def test_mixed_split_radius_error(M, split_radius, bound):
    """The mixed form evaluates pairs beyond the split radius in FP32 (default
    1.5 sigma) and closer pairs in double-float; a split radius at the list
    radius keeps every pair in double-float.  Force error against FP64 on the
    same positions, per atom, floored at 0.1 of the RMS force."""
    pos, L = fcc(8)
    vel = mb_velocities(len(pos), 0.728, 4)
    ref = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64)
    ref.run(150)
    p, v, _ = ref.state()
    mix = M.LJSystem(p, v, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED, split_radius=split_radius)
    ref.set_state(p, v)
    em, wm = mix.eval_forces()
    er, wr = ref.eval_forces()
    _, _, fm = mix.state()
    _, _, fr = ref.state()
    err = per_atom_rel_err(fm, fr, 0.1)
    assert err < bound, err
    assert abs(em - er) <= 1e-9 * abs(er) and abs(wm - wr) <= 1e-9 * abs(wr)
    assert mix.stats()["pairs"] > 1.9 * ref.stats()["pairs"]


def test_elongated_box_linear_sort_fallback(M):
    """A box of more than 1024 cells along x: the Z-order key needs more than
    10 bits per axis, so the stepper sorts by row-major cells instead; forces
    still match the FP64 form, and a short run stays finite."""
    rng = np.random.default_rng(17)
    box = np.array([1500.0, 6.0, 6.0])
    # a dilute gas on a jittered lattice (no close contacts)
    g = np.stack(np.meshgrid(np.arange(0.75, 1500.0, 1.5), np.arange(0.75, 6.0, 1.5),
                             np.arange(0.75, 6.0, 1.5), indexing="ij"), -1).reshape(-1, 3)
    pos = g + rng.uniform(-0.2, 0.2, g.shape)
    vel = rng.normal(0, 0.5, pos.shape)
    ref = M.LJSystem(pos, vel, [0, 0, 0], box, precision=M.PREC_FP64)
    er, _ = ref.eval_forces()
    _, _, fr = ref.state()
    rms = np.sqrt((fr * fr).sum(1).mean())
    # every pair in double-float: the sort fallback alone
    dfl = M.LJSystem(pos, vel, [0, 0, 0], box, precision=M.PREC_MIXED, split_radius=2.8)
    em, _ = dfl.eval_forces()
    _, _, fm = dfl.state()
    assert np.abs(fm - fr).max() / rms < 1e-8
    assert abs(em - er) <= 1e-7 * abs(er)
    # the default split: this near-lattice gas has a small RMS force (about 1.6
    # against 13.7 in the dense fluid) and almost all of its pairs beyond the
    # split radius, in FP32.  Relative to the RMS force the error stays below
    # 1e-6; per atom, floored at 0.1 of the (small) RMS force, it is the FP32
    # far-pair limit, about 1.4e-6, and a larger split radius (1.8 sigma)
    # brings it below 1e-6
    mix = M.LJSystem(pos, vel, [0, 0, 0], box, precision=M.PREC_MIXED)
    mix.eval_forces()
    _, _, fm = mix.state()
    assert np.abs(fm - fr).max() / rms < 1e-6
    assert per_atom_rel_err(fm, fr, 0.1) < 2e-6
    wide = M.LJSystem(pos, vel, [0, 0, 0], box, precision=M.PREC_MIXED, split_radius=1.8)
    wide.eval_forces()
    assert per_atom_rel_err(wide.state()[2], fr, 0.1) < 1e-6
    e = mix.run(30)
    assert np.all(np.isfinite(e))


def test_one_pass_and_two_kernel_tile_builds_agree(M):
    """The tile list built in one pass from the cell list and the one made
    from the int32 rows (tile_build="two_kernel"): the same pairs in the same
    rows and order, so the forces and a short trajectory are bitwise equal."""
    pos, L = fcc(16)  # 16,384 atoms
    vel = mb_velocities(len(pos), 0.728, 9)
    a = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED)
    b = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED, tile_build="two_kernel")
    a.run(35)
    b.run(35)
    assert a.tile_stats()["tiled"] and b.tile_stats()["tiled"]
    assert a.tile_stats()["two_pass_builds"] == 0
    for x, y in zip(a.state(), b.state()):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a.pair_keys(), b.pair_keys())


def test_unsorted_atoms_take_the_two_kernel_tile_build(M):
    """Atoms never cell-sorted and given in random order: a tile's rows are
    scattered through the box, so the one-pass tile build overflows its span
    table and the rebuild makes the int32 rows and their tile form instead.
    The tile form it makes holds the same pairs in the same order (forces
    bitwise equal to the gather form, which reads the int32 rows directly)."""
    pos, L = fcc(12)  # 6,912 atoms
    rng = np.random.default_rng(11)
    perm = rng.permutation(len(pos))
    pos = pos[perm] + rng.normal(0, 0.05, pos.shape)
    vel = mb_velocities(len(pos), 0.728, 5)
    t = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED, sort_atoms=0)
    g = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED, sort_atoms=0, gather_neighbours=True)
    t.eval_forces()
    g.eval_forces()
    st = t.tile_stats()
    assert st["two_pass_builds"] >= 1 and st["unfit_tiles"] > 0
    np.testing.assert_array_equal(t.state()[2], g.state()[2])
    np.testing.assert_array_equal(t.pair_keys(), g.pair_keys())
    t.run(20)
    g.run(20)
    np.testing.assert_array_equal(t.state()[0], g.state()[0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_state_reported_by_the_stepper(M, precision):
    """An infinite velocity, set on the host, makes a position infinite after
    the first drift; the stepper reports MRMD_ERR_NONFINITE at the next list
    rebuild (every 10 steps), within the same run call."""
    prec = M.PREC_FP64 if precision == "fp64" else M.PREC_MIXED
    pos, L = fcc(6)
    vel = mb_velocities(len(pos), 0.728, 9)
    vel[100, 0] = np.inf
    s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=prec)
    with pytest.raises(M.MrmdError) as ei:
        s.run(25)
    assert ei.value.code == -4
    # a NaN position fails at the first build
    pos2 = pos.copy()
    pos2[7, 2] = np.nan
    s2 = M.LJSystem(pos2, mb_velocities(len(pos), 0.728, 9), [0, 0, 0], [L] * 3, precision=prec)
    with pytest.raises(M.MrmdError) as ei:
        s2.run(1)
    assert ei.value.code == -4


def espp_oracle(orc, espp, shifted=True):
    """Oracle half list (canonical pair keys) and FP64 forces of the ESPP
    system (tests/LennardJones/positions.txt of the reference)."""
    g, pos = espp
    L, rc, skin = g["box"], g["rc"], g["skin"]
    sd = orc.subdomain([0, 0, 0], [L] * 3, rc + skin)
    ao = orc.Atoms.from_positions(pos, capacity=60000)
    corr = orc.create_ghosts(ao, sd)
    co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd.minGhostCorner,
                                 sd.maxGhostCorner, 1.0, 64)
    keys = orc.canonical_pairs(co, no, corr, ao.numLocal)
    ao.force[:] = 0
    E, W = orc.lj_apply(orc.lj_table(0.0, rc, 1.0, 1.0, 1, shifted), rc * rc, ao, co, no)
    orc.ghost_to_real(ao, corr)
    return pos, L, keys, ao.force[: ao.numLocal].copy(), E, W


@pytest.mark.parametrize("form", ["fp64", "mixed", "mixed_gather"])
def test_stepper_list_is_the_oracle_pair_set(M, orc, espp, form):
    """The list the stepper's pair kernel reads (the FP64 half list; the mixed
    form's near + far full list, decoded from its shared-memory tiles or from
    the int32 lists), mapped to unordered pairs of original atom indices, is
    the oracle's half-list pair set bit for bit: once per pair in the half
    list, twice in the full list."""
    pos, L, ko, _, _, _ = espp_oracle(orc, espp)
    prec = M.PREC_FP64 if form == "fp64" else M.PREC_MIXED
    s = M.LJSystem(pos, np.zeros_like(pos), [0, 0, 0], [L] * 3, precision=prec,
                   gather_neighbours=form == "mixed_gather")
    s.eval_forces()
    kg = s.pair_keys()
    if form == "fp64":
        np.testing.assert_array_equal(kg, ko)
    else:
        assert len(kg) == 2 * len(ko)
        np.testing.assert_array_equal(kg[0::2], ko)
        np.testing.assert_array_equal(kg[1::2], ko)
        assert s.tile_stats()["tiled"] == (form == "mixed")


def test_mixed_tile_forces_per_atom_against_oracle(M, orc, espp):
    """Mixed form on the ESPP system against the oracle's FP64 forces, per atom:
    |dF_i| <= 1e-6 max(|F_i|, 0.1 rms|F|); the tile and the gather form read the
    same records in the same order and agree bitwise; energy and virial
    (double-float sums of u^3 and u^6) within 1e-9 relative."""
    pos, L, _, fo, Eo, Wo = espp_oracle(orc, espp)
    vel = np.zeros_like(pos)
    t = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED)
    g = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_MIXED, gather_neighbours=True)
    et, wt = t.eval_forces()
    eg, wg = g.eval_forces()
    ft, fg = t.state()[2], g.state()[2]
    assert t.tile_stats()["tiled"] and not g.tile_stats()["tiled"]
    np.testing.assert_array_equal(ft, fg)
    err = per_atom_rel_err(ft, fo, 0.1)
    assert err <= 1e-6, err
    assert abs(et - Eo) <= 1e-9 * abs(Eo) and abs(wt - Wo) <= 1e-9 * abs(Wo), (et, Eo, wt, Wo)
    assert abs(et - eg) <= 1e-12 * abs(et)
