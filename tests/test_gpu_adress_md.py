"""The fused AdResS stepper against an oracle-driven loop of the same actions
(LJ_IdealGas, Langevin, UpdateMolecules/Slab, ContributeMoleculeForceToAtoms,
MultiResGhostLayer, ThermodynamicForce sample/apply/update)."""
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


def system(n, box, seed):
    return random_system(n, box, seed)


def gpu_system(M, pos, vel, box, p, precision, graph=True, composed=False):
    return M.AdResSSystem(pos, vel, [0, 0, 0], box, [box[0] / 2, box[1] / 2, box[2] / 2], p["at"], p["hy"],
                          p["nu"], rc=p["rc"], skin=p["skin"], sigma=p["sigma"], epsilon=p["epsilon"],
                          capping_distance=p["cap"], precision=precision, dt=p["dt"], rebuild_interval=p["K"],
                          gamma=p["gamma"], temperature=p["T"], seed=p["seed"], tf=True, tf_bin_width=p["binw"],
                          tf_target_density=p["rho"], tf_modulation=p["mod"], tf_sigma=p["tfs"],
                          tf_range=p["tfr"], tf_sample_interval=p["S"], tf_update_interval=p["U"],
                          use_graph=graph, composed=composed)


@pytest.mark.parametrize("graph,composed", [(False, False), (True, False), (False, True), (True, True)])
def test_adress_trajectory_matches_oracle(M, orc, graph, composed):
    """Both engines of the stepper (the batched engine with one replica, the
    default for unit masses, and the composed actions) against the oracle."""
    box = [36.0, 10.0, 10.0]
    pos, vel = system(1800, box, 5)
    steps = 13
    po, vo, eo, fo, _ = oracle_loop(orc, pos, vel, box, steps, P)
    s = gpu_system(M, pos, vel, box, P, M.PREC_FP64, graph, composed)
    eg = s.run(steps)
    pg, vg, _ = s.state()
    # Langevin noise and the Slab weights go through exp/log/cos/sin, which may
    # differ by ulps between host and device libraries
    np.testing.assert_allclose(pg, po, rtol=0, atol=1e-9)
    np.testing.assert_allclose(vg, vo, rtol=0, atol=1e-8)
    np.testing.assert_allclose(eg, eo, rtol=1e-9)
    fg, _ = s.thermodynamic_force()
    np.testing.assert_allclose(fg, fo, rtol=1e-9, atol=1e-12)
    st = s.stats()
    assert st["steps"] == steps and st["rebuilds"] == 3 and st["ghost_molecules"] > 0


@pytest.mark.parametrize("composed", [False, True])
def test_adress_mixed_close_to_fp64(M, composed):
    box = [36.0, 10.0, 10.0]
    pos, vel = system(1800, box, 6)
    a = gpu_system(M, pos, vel, box, P, M.PREC_FP64, composed=composed)
    b = gpu_system(M, pos, vel, box, P, M.PREC_MIXED, composed=composed)
    ea = a.run(6)
    eb = b.run(6)
    pa, va, _ = a.state()
    pb, vb, _ = b.state()
    np.testing.assert_allclose(eb, ea, rtol=1e-6)
    # the mixed form evaluates pair energies in FP32 and the AdResS drift force
    # (-V_ij/2 grad lambda) uses them; on this random start (capped forces of
    # 1000 sigma/eps) six steps move positions by < 1e-7
    assert np.abs(pa - pb).max() < 1e-7


# The 34,560-molecule AdResS workload: single-site molecules in 120 x 24 x 24,
# density 0.5, capped LJ (cap 1000 <-> r_cap 0.7842), atomistic slab 30,
# hybrid 10, Langevin T 1 gamma 1, thermodynamic force on 100 bins sampled
# every step and updated every 1,000 steps
ADRESS_34560 = dict(rc=2.5, skin=0.3, sigma=1.0, epsilon=1.0, cap=0.7842, dt=0.005, K=10, gamma=1.0, T=1.0, seed=77,
               at=30.0, hy=10.0, nu=1, binw=1.2, rho=0.5, mod=1.0, tfs=2.4, tfr=3.0, S=1, U=1000)


def test_adress_34560_thermodynamic_force_over_update_cycles(M, orc):
    """Three thermodynamic-force update cycles (ThermodynamicForce.hpp:124-152,
    every 1,000 steps) of the 34,560-molecule system, then 990 steps into the
    fourth, on the GPU (FP64 form) and in the oracle loop from the same start
    with the same noise.  Over thousands of steps the two trajectories
    separate (chaos amplifies the last bits of the summation order), so the
    table and the density profile are compared statistically.

    Tolerance: the spread of two independent realizations, measured by a
    second GPU run with another noise seed.  With s = the root mean square
    over bins of (GPU seed A - GPU seed B), which estimates the standard
    deviation of the difference of two realizations, the GPU - oracle
    difference (same seed A; after thousands of steps as different as two
    realizations) must satisfy rms <= 1.6 s (the rms of 100 smoothed,
    correlated bins is uncertain to about 25%) and max over bins <= 4.5 s
    (4.5 standard deviations).  Both for the table after the third update
    and for the density profile of the fourth cycle (counts per sample)."""
    p = ADRESS_34560
    box = [120.0, 24.0, 24.0]
    pos, vel = system(34560, box, 11)
    steps = 3 * p["U"] + 990
    orc.set_threads(orc.max_threads())
    tf_out = {}
    _, _, _, fo, _ = oracle_loop(orc, pos, vel, box, steps, p, tf_out=tf_out)
    assert tf_out["samples"] == 990
    res = []
    for seed in (p["seed"], p["seed"] + 1000):
        s = gpu_system(M, pos, vel, box, dict(p, seed=seed), M.PREC_FP64)
        s.run(steps, energies=False)
        f, d = s.thermodynamic_force()
        res.append((f, d / 990.0))
        s.close()
    do = tf_out["density"] / 990.0
    for name, (ga, gb), o in (("table", (res[0][0], res[1][0]), fo), ("density", (res[0][1], res[1][1]), do)):
        spread = float(np.sqrt(np.mean((ga - gb) ** 2)))
        diff = ga - o
        assert spread > 0.0, name
        assert float(np.sqrt(np.mean(diff ** 2))) <= 1.6 * spread, (name, diff, spread)
        assert float(np.abs(diff).max()) <= 4.5 * spread, (name, np.abs(diff).max(), spread)
    # the table moved away from zero: three updates did act
    assert float(np.abs(fo).max()) > 3.0 * float(np.sqrt(np.mean((res[0][0] - res[1][0]) ** 2)))
