"""Batched AdResS replicas (mrmd_batch_*): one replica against the
oracle-driven AdResS loop, every replica of a batch bitwise against the same
replica run alone, the three list layouts (rows, near/far rows, 8 x 4
cluster pairs), capacity overflow recovery, and the autotuner."""
import numpy as np
import pytest

from tests.adress_loop import oracle_loop, random_system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


P = dict(rc=2.5, skin=0.3, sigma=1.0, epsilon=1.0, cap=0.7842, dt=0.005, K=5, gamma=1.0, T=1.0, seed=77,
         at=10.0, hy=5.0, nu=1, binw=1.2, rho=0.5, mod=1.0, tfs=2.4, tfr=3.0, S=2, U=6)


def batch(M, replicas, pos, vel, p=P, precision=None, **tuning):
    kw = dict(threads_per_row=1, block_size=128, rebuild_interval=p["K"], sort_every=0, graph_steps=p["K"])
    kw.update(tuning)
    if kw.get("list_layout") == 2:
        kw["threads_per_row"] = 4  # the cluster layout's 4 lanes per row
    return M.BatchSystem(replicas, pos, vel, hybrid_diameter=p["hy"], nu=p["nu"], rc=p["rc"], skin=p["skin"],
                         sigma=p["sigma"], epsilon=p["epsilon"], capping_distance=p["cap"],
                         precision=M.PREC_FP64 if precision is None else precision, dt=p["dt"],
                         gamma=p["gamma"], temperature=p["T"], tf=True, tf_bin_width=p["binw"],
                         tf_target_density=p["rho"], tf_modulation=p["mod"], tf_sigma=p["tfs"], tf_range=p["tfr"],
                         tf_sample_interval=p["S"], tf_update_interval=p["U"], **kw)


def replica(M, n, box, at, seed, center=None):
    c = center if center is not None else [box[0] / 2, box[1] / 2, box[2] / 2]
    return M.Replica(n, [0, 0, 0], box, c, at, seed)


@pytest.mark.parametrize("graph,layout", [(0, 0), (5, 0), (5, 2)])
def test_single_replica_matches_oracle(M, orc, graph, layout):
    box = [36.0, 10.0, 10.0]
    pos, vel = random_system(1800, box, 5)
    steps = 13
    po, vo, eo, fo, mo = oracle_loop(orc, pos, vel, box, steps, P)
    b = batch(M, [replica(M, 1800, box, P["at"], P["seed"])], pos, vel, graph_steps=graph, list_layout=layout)
    eg = b.run(steps)[:, 0]
    pg, vg, _ = b.state()
    # the compensation histogram is accumulated in 2^-32 fixed point and the
    # Langevin noise goes through exp/log/cos/sin (host vs device ulps)
    np.testing.assert_allclose(pg, po, rtol=0, atol=1e-9)
    np.testing.assert_allclose(vg, vo, rtol=0, atol=1e-8)
    np.testing.assert_allclose(eg, eo, rtol=1e-9)
    fg, _ = b.thermodynamic_force()
    np.testing.assert_allclose(fg[0], fo, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(b.compensation()[0], mo, rtol=1e-8, atol=1e-8)
    st = b.stats()
    assert st["steps"] == steps and st["rebuilds"] == 3 and st["ghost_molecules"] > 0
    assert st["flags"] & 3 == 0


def test_slab_reaching_into_the_ghost_layer_matches_oracle(M, orc):
    """A box whose slab extends past the ghost layer: the weights of a pair
    with a ghost differ between its two periodic instances, and the batch
    must use the instance Cabana's half list keeps."""
    box = [12.0, 9.0, 9.0]
    p = dict(P, at=4.0, hy=5.0)
    n = int(0.5 * 12 * 9 * 9)
    pos, vel = random_system(n, box, 9)
    steps = 11
    po, vo, eo, fo, mo = oracle_loop(orc, pos, vel, box, steps, p)
    for prec, layout, tol, etol in ((M.PREC_FP64, 0, 1e-9, 1e-9), (M.PREC_FP64, 2, 1e-9, 1e-9),
                                    (M.PREC_MIXED, 0, 1e-6, 1e-5), (M.PREC_MIXED, 1, 1e-6, 1e-5),
                                    (M.PREC_MIXED, 2, 1e-6, 1e-5)):
        b = batch(M, [replica(M, n, box, p["at"], p["seed"])], pos, vel, p=p, precision=prec,
                  list_layout=layout)
        eg = b.run(steps)[:, 0]
        pg, vg, _ = b.state()
        np.testing.assert_allclose(pg, po, rtol=0, atol=tol)
        np.testing.assert_allclose(eg, eo, rtol=etol)


def replica_set(M):
    rng = np.random.default_rng(3)
    reps, P_, V_ = [], [], []
    specs = [(350, 4.5), (900, 9.0), (1700, 16.0), (2600, 24.0), (5200, 44.0)]
    for k, (n, lx) in enumerate(specs):
        box = [lx, 12.0, 12.0] if k % 2 else [lx, 14.0, 12.0]
        at = float(rng.uniform(4.0, 14.0))
        reps.append(replica(M, n, box, at, 1000 + k))
        p, v = random_system(n, box, 40 + k)
        P_.append(p)
        V_.append(v)
    return reps, np.concatenate(P_), np.concatenate(V_)


@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_split", "fp64_cluster", "mixed_cluster"])
def test_replicas_bitwise_equal_alone(M, prec):
    """Clusters are aligned to each replica's first molecule and first cell,
    so the cluster layout keeps every replica's pair order too."""
    precision = M.PREC_FP64 if prec.startswith("fp64") else M.PREC_MIXED
    reps, pos, vel = replica_set(M)
    layout = 1 if prec == "mixed_split" else (2 if prec.endswith("cluster") else 0)
    tune = dict(threads_per_row=4 if layout == 2 else 2, block_size=128, rebuild_interval=5, sort_every=2,
                graph_steps=10, list_layout=layout)
    b = batch(M, reps, pos, vel, precision=precision, **tune)
    steps = 23
    eb = b.run(steps)
    pb, vb, fb = b.state()
    assert b.stats()["graph_launches"] == 2
    for r, rep in enumerate(reps):
        sl = b.replica_slice(r)
        a = batch(M, [rep], pos[sl], vel[sl], precision=precision, **tune)
        ea = a.run(steps)[:, 0]
        pa, va, fa = a.state()
        assert np.array_equal(pa, pb[sl]), f"replica {r} positions"
        assert np.array_equal(va, vb[sl]), f"replica {r} velocities"
        assert np.array_equal(fa, fb[sl]), f"replica {r} forces"
        # energies are diagnostics summed with atomics (FP32 warp sums in the
        # mixed form), so they agree to rounding, not bitwise
        np.testing.assert_allclose(eb[:, r], ea, rtol=1e-11 if precision == M.PREC_FP64 else 1e-5, atol=1e-9)
        ta, _ = a.thermodynamic_force()
        tb, _ = b.thermodynamic_force()
        assert np.array_equal(ta[0], tb[r])


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_mixed_close_to_fp64(M, layout):
    """Layouts 1 and 2 evaluate the pairs beyond 1.4 sigma in FP32."""
    reps, pos, vel = replica_set(M)
    a = batch(M, reps, pos, vel, precision=M.PREC_FP64)
    b = batch(M, reps, pos, vel, precision=M.PREC_MIXED, list_layout=layout)
    # the first step's forces act on identical positions (the pre-force
    # integration is FP64 in both forms)
    a.run(1)
    b.run(1)
    pa, _, fa = a.state()
    pb, _, fb = b.state()
    assert np.array_equal(pa, pb)
    rms = np.sqrt((fa ** 2).sum(axis=1).mean())
    assert np.abs(fa - fb).max() / rms < 1e-6
    a.run(5)
    b.run(5)
    pa, _, _ = a.state()
    pb, _, _ = b.state()
    assert np.abs(pa - pb).max() < 1e-7


@pytest.mark.parametrize("prec,layout", [("fp64", 0), ("mixed", 1), ("fp64", 2), ("mixed", 2)])
def test_capacity_overflow_recovery(M, prec, layout):
    """Ghost and list buffers that start far too small (near and far rows in
    the split layout, cluster-pair rows in the cluster layout) grow by
    roll-back and re-run, bitwise like a batch that never overflowed."""
    precision = M.PREC_FP64 if prec == "fp64" else M.PREC_MIXED
    reps, pos, vel = replica_set(M)
    tune = dict(rebuild_interval=5, sort_every=1, graph_steps=10, list_layout=layout)
    a = batch(M, reps, pos, vel, precision=precision, **tune)
    b = M.BatchSystem(reps, pos, vel, hybrid_diameter=P["hy"], rc=P["rc"], skin=P["skin"],
                      capping_distance=P["cap"], dt=P["dt"], tf_sample_interval=P["S"], tf_update_interval=P["U"],
                      precision=precision, threads_per_row=4 if layout == 2 else 1, block_size=128,
                      rebuild_interval=5, sort_every=1,
                      graph_steps=10, list_layout=layout, initial_max_neighbors=6, initial_ghost_capacity=32)
    a.run(20)
    b.run(20)
    assert b.stats()["recoveries"] >= 1
    pa, va, _ = a.state()
    pb, vb, _ = b.state()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)


def test_autotune_picks_a_candidate_and_keeps_the_state(M):
    reps, pos, vel = replica_set(M)
    b = batch(M, reps, pos, vel, rebuild_interval=5, sort_every=1, graph_steps=10)
    b.run(10)
    p0, v0, _ = b.state()
    best, trials = b.autotune(trial_steps=10)
    assert best in [t for t, _ in trials]
    assert any(ms is not None for _, ms in trials)
    p1, v1, _ = b.state()
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
    assert b.stats()["steps"] == 10
    b.run(20)
    assert b.stats()["steps"] == 30


def test_cluster_layout_lists_the_same_pairs(M):
    """The 8 x 4 cluster rows hold exactly the pairs of the per-molecule rows
    (the same tests per pair), and the FP64 forces of the two layouts differ
    only by the order of the pair sums."""
    reps, pos, vel = replica_set(M)
    a = batch(M, reps, pos, vel, sort_every=1)
    b = batch(M, reps, pos, vel, sort_every=1, list_layout=2)
    a.run(1)
    b.run(1)
    la, lb = a.list_stats(), b.list_stats()
    assert la["pairs"] == lb["pairs"] > 0
    assert la["slots_per_entry"] == 1 and lb["slots_per_entry"] == 32
    assert 0.0 < lb["lane_efficiency"] <= 1.0
    _, _, fa = a.state()
    _, _, fb = b.state()
    rms = np.sqrt((fa ** 2).sum(axis=1).mean())
    assert np.abs(fa - fb).max() / rms < 1e-12
    a.run(9)
    b.run(9)
    assert a.list_stats()["pairs"] == b.list_stats()["pairs"]


@pytest.mark.parametrize("layout,prec", [(0, "fp64"), (1, "mixed"), (2, "fp64"), (2, "mixed")])
def test_batch_lists_are_the_oracle_pair_set(M, orc, layout, prec):
    """Each replica's list of the batch engine (per-molecule rows, near/far
    rows, 8 x 4 cluster pairs), mapped to unordered pairs of the replica's
    molecules, against the oracle's half list of the same positions.
    Replica 0's slab reaches past its box, so no pair is pruned and the two
    pair sets are equal bit for bit.  Replica 1 has a narrow slab: pairs of two
    molecules that stay coarse grained until the next rebuild (|x - c| beyond
    r_at/2 + d_hy + skin + 1e-3, decided in FP32) are left out.  There the list
    is a subset of the oracle's, holds every pair with a molecule 1e-4 inside
    that bound, and no pair with both molecules r_list + 1e-4 beyond it.  No
    pair appears more than twice (the full list's two rows)."""
    rc, skin, hy = P["rc"], P["skin"], P["hy"]
    specs = [([20.0, 12.0, 12.0], 16.0, 700, 11), ([44.0, 12.0, 14.0], 6.0, 1300, 12)]
    reps, pos, vel = [], [], []
    for box, at, n, seed in specs:
        reps.append(replica(M, n, box, at, 500 + seed))
        p_, v_ = random_system(n, box, seed)
        pos.append(p_)
        vel.append(v_)
    precision = M.PREC_MIXED if prec == "mixed" else M.PREC_FP64
    b = batch(M, reps, np.concatenate(pos), np.concatenate(vel), precision=precision, list_layout=layout,
              sort_every=1)
    b.run(1)  # the first step rebuilds at its drifted positions and keeps them
    state = b.state()[0]
    off = 0
    for r, (box, at, n, _) in enumerate(specs):
        p_ = state[off:off + n]
        off += n
        sd = orc.subdomain([0, 0, 0], box, rc + skin)
        ao = orc.Atoms.from_positions(p_, capacity=8 * n)
        corr = orc.create_ghosts(ao, sd)
        co, no = orc.build_half_list(ao.pos, ao.n, 0, ao.numLocal, rc + skin, sd.minGhostCorner,
                                     sd.maxGhostCorner, 1.0, 256)
        ko = orc.canonical_pairs(co, no, corr, ao.numLocal)
        kb_all = b.pair_keys(r)
        kb, mult = np.unique(kb_all, return_counts=True)
        assert mult.max() <= 2
        if r == 0:
            np.testing.assert_array_equal(kb, ko)
            continue
        assert np.isin(kb, ko).all()
        deep = at / 2 + hy + skin + 1e-3
        a_, c_ = ko >> 32, ko & 0xffffffff
        dmin = np.minimum(np.abs(p_[a_, 0] - box[0] / 2), np.abs(p_[c_, 0] - box[0] / 2))
        inb = np.isin(ko, kb)
        assert inb[dmin < deep - 1e-4].all()
        pruned = dmin > deep + rc + skin + 1e-4
        assert pruned.sum() > 100 and not inb[pruned].any()


@pytest.mark.parametrize("prec,layout,tpr", [("fp64", 0, 2), ("mixed", 1, 1), ("mixed", 2, 4)])
def test_persistent_steps_bitwise_equal(M, prec, layout, tpr):
    """The steps between rebuilds as one persistent cooperative launch (grid
    barriers between the phases) against one launch per phase, inside the same
    CUDA graphs: positions, velocities and forces bitwise equal (every
    molecule, ghost, row and replica does the same arithmetic), energies to
    the order of the per-replica atomic sums, the same TF tables."""
    reps, pos, vel = replica_set(M)
    precision = M.PREC_MIXED if prec == "mixed" else M.PREC_FP64
    tune = dict(threads_per_row=tpr, block_size=128, rebuild_interval=5, sort_every=2, graph_steps=10,
                list_layout=layout)
    a = batch(M, reps, pos, vel, precision=precision, **tune)
    b = batch(M, reps, pos, vel, precision=precision, persistent=True, **tune)
    assert b.tuning["persistent"] == 1 and a.tuning["persistent"] == 0
    ea = a.run(30)
    eb = b.run(30)
    for x, y in zip(a.state(), b.state()):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_allclose(eb, ea, rtol=1e-12, atol=1e-9)
    for ta, tb in zip(a.thermodynamic_force()[0], b.thermodynamic_force()[0]):
        np.testing.assert_array_equal(ta, tb)
    assert b.stats()["steps"] == 30


def test_grid_barrier_time_limit(M):
    """The persistent kernel's grid barrier gives up after its time limit:
    with one block that never arrives the others stop waiting after 50 ms and
    the call returns MRMD_ERR_TIMEOUT; the context keeps working."""
    assert M.grid_sync_selftest(rounds=1000) == 0
    assert M.grid_sync_selftest(rounds=10, skip_block=0, limit_ms=50.0) == -5
    assert M.grid_sync_selftest(rounds=1000) == 0


def test_layout_switch_and_bad_cluster_tuning(M):
    """Switching layouts between runs keeps the trajectory on the FP64 path
    (to rounding), and the cluster layout takes 4 lanes per row only."""
    reps, pos, vel = replica_set(M)
    a = batch(M, reps, pos, vel)
    b = batch(M, reps, pos, vel)
    a.run(10)
    b.run(5)
    b.tuning = dict(list_layout=2, threads_per_row=4)
    b.run(5)
    assert b.tuning["list_layout"] == 2
    pa, _, _ = a.state()
    pb, _, _ = b.state()
    assert np.abs(pa - pb).max() < 1e-10
    with pytest.raises(M.MrmdError):
        b.tuning = dict(list_layout=2, threads_per_row=2)
    with pytest.raises(M.MrmdError):
        b.tuning = dict(list_layout=3, threads_per_row=4)
