"""Adjoint of the AdResS trajectory (mrmd_diff_*): one force evaluation's
vector-Jacobian product against central finite differences, the trajectory
gradient against central finite differences of the GPU loss and of the
oracle's (CPU FP64) loss, the torch.autograd shim, a gradient-descent step on
the thermodynamic-force table, and the table fit by gradient descent next to
the reference's iterative update."""
import numpy as np
import pytest

from tests.adress_loop import oracle_loop, random_system

pytestmark = pytest.mark.gpu

BOX = [40.0, 10.0, 10.0]
AT, HY = 10.0, 5.0
P = dict(rc=2.5, skin=0.3, sigma=1.0, epsilon=1.0, cap=0.7842, dt=0.005, K=5, gamma=1.0, T=1.0, seed=31,
         at=AT, hy=HY, nu=1, binw=1.2, rho=0.5, mod=1.0, tfs=1.0, tfr=1.0, S=1, U=10 ** 6)


@pytest.fixture(scope="module")
def M():
    import mrmd_gb300 as M

    M.default_context()
    return M


def system(M, n=2000, steps=12, window=6, ckpt=5, bins=32, seed=3, precision=None):
    pos, vel = random_system(n, BOX, seed)
    rep = M.Replica(n, [0, 0, 0], BOX, [BOX[0] / 2, BOX[1] / 2, BOX[2] / 2], AT, P["seed"])
    d = M.DiffSystem(rep, pos, vel, hybrid_diameter=HY, steps=steps, window=window, checkpoint_interval=ckpt,
                     loss_bins=bins, loss_sigma=1.0, capping_distance=P["cap"], rebuild_interval=5,
                     precision=M.PREC_FP64 if precision is None else precision)
    return d, pos, vel


def table_of(d, seed=1, scale=0.5):
    return np.random.default_rng(seed).normal(0.0, scale, d.num_bins)


def test_force_vjp_matches_finite_differences(M):
    d, pos, vel = system(M, steps=5, window=5, ckpt=5)
    tab = table_of(d)
    rng = np.random.default_rng(7)
    a = rng.normal(size=(d.n, 3))
    f0, xbar, gt, ge, gs = d.force_vjp(tab, 1.0, 1.0, a)
    # central differences of Phi = sum a.F, formed as sum a.(F+ - F-): the
    # force differences vanish except near the moved molecule, so the rounding
    # of the two large sums Phi(x +- h) does not enter
    dphi = lambda fp, fm: float((a * (fp - fm)).sum())
    # molecules in the hybrid region exercise the weight and drift terms
    x = pos[:, 0]
    hybrid = np.nonzero((np.abs(x - BOX[0] / 2) > AT / 2 + 0.2) & (np.abs(x - BOX[0] / 2) < AT / 2 + HY - 0.2))[0]
    h = 1e-6
    for k in list(hybrid[:4]) + [0]:
        for ax in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[k, ax] += h
            pm[k, ax] -= h
            d.set_state(pp, vel)
            fp = d.force_vjp(tab, 1.0, 1.0, a)[0]
            d.set_state(pm, vel)
            fm = d.force_vjp(tab, 1.0, 1.0, a)[0]
            fd = dphi(fp, fm) / (2 * h)
            assert abs(fd - xbar[k, ax]) <= 1e-6 * max(1.0, abs(fd)), (k, ax, fd, xbar[k, ax])
    d.set_state(pos, vel)
    for which, g in (("eps", ge), ("sig", gs)):
        args_p = (1.0 + h, 1.0) if which == "eps" else (1.0, 1.0 + h)
        args_m = (1.0 - h, 1.0) if which == "eps" else (1.0, 1.0 - h)
        fd = dphi(d.force_vjp(tab, *args_p, a)[0], d.force_vjp(tab, *args_m, a)[0]) / (2 * h)
        assert abs(fd - g) <= 1e-6 * max(1.0, abs(fd)), (which, fd, g)
    # the table enters linearly: dPhi/dT_b = sum of a_x over molecules in bin b
    for b in (0, d.num_bins // 2, d.num_bins - 1):
        tp, tm = tab.copy(), tab.copy()
        tp[b] += 1.0
        tm[b] -= 1.0
        fd = dphi(d.force_vjp(tp, 1.0, 1.0, a)[0], d.force_vjp(tm, 1.0, 1.0, a)[0]) / 2.0
        assert abs(fd - gt[b]) <= 1e-9 * max(1.0, abs(fd)), (b, fd, gt[b])


def central_fd(f, x0, h):
    return (f(x0 + h) - f(x0 - h)) / (2 * h)


def test_trajectory_gradient_matches_finite_differences(M):
    d, pos, vel = system(M)
    tab = table_of(d, seed=2, scale=0.3)
    L0 = d.forward(tab, 1.0, 1.0)
    gt, ge, gs = d.backward()
    h = 1e-6
    # the loss is summed with FP64 atomics (order-dependent rounding, ~1e-15 L),
    # which central differences amplify by 1/h: that is the noise floor
    floor = 1e-15 * abs(L0) / h * 10
    fe = central_fd(lambda e: d.forward(tab, e, 1.0), 1.0, h)
    fs = central_fd(lambda s: d.forward(tab, 1.0, s), 1.0, h)
    assert abs(fe - ge) <= 1e-6 * abs(fe) + floor, (fe, ge)
    assert abs(fs - gs) <= 1e-6 * abs(fs) + floor, (fs, gs)
    for b in np.argsort(-np.abs(gt))[:3]:
        def Lb(v, b=b):
            t = tab.copy()
            t[b] = v
            return d.forward(t, 1.0, 1.0)
        fb = central_fd(Lb, tab[b], h)
        assert abs(fb - gt[b]) <= 1e-6 * abs(fb) + floor, (b, fb, gt[b])


def oracle_loss(orc, pos, vel, tab, eps, sig, steps, window, bins, lsig=1.0):
    p = dict(P, epsilon=eps, sigma=sig)
    n = len(pos)
    Lx, area = BOX[0], BOX[1] * BOX[2]
    centres = (np.arange(bins) + 0.5) * (Lx / bins)
    rho = np.zeros(bins)
    norm = 1.0 / (np.sqrt(2 * np.pi) * lsig)

    def on_step(st, x):
        if st < steps - window:
            return
        dd = x[:, 0][:, None] - centres[None, :]
        dd -= Lx * np.rint(dd / Lx)
        k = norm * np.exp(-0.5 * dd * dd / lsig ** 2)
        k[np.abs(dd) > 6 * lsig] = 0.0
        rho[:] += k.sum(axis=0)

    oracle_loop(orc, pos, vel, BOX, steps, p, tf_table=tab, comp_frozen=True, on_step=on_step)
    r = rho / (window * area)
    return float(((r - n / (Lx * area)) ** 2).sum())


def test_trajectory_gradient_matches_oracle_finite_differences(M, orc):
    """The CPU FP64 reference: central differences of the oracle loop's loss.
    The loss is only piecewise smooth (the LJ force jumps at the cutoff, the
    TF table is piecewise constant in x): on this instance a kink lies within
    1e-6 of sigma = 1, so the differences take h = 1e-7.  The GPU and oracle
    trajectories agree to ~1e-15, far below what 1/h amplifies."""
    steps, window, bins = 10, 5, 32
    d, pos, vel = system(M, steps=steps, window=window, ckpt=5, bins=bins)
    tab = table_of(d, seed=4, scale=0.3)
    L = d.forward(tab, 1.0, 1.0)
    Lo = oracle_loss(orc, pos, vel, tab, 1.0, 1.0, steps, window, bins)
    print("GPU vs oracle loss (relative):", abs(L - Lo) / abs(Lo))
    assert abs(L - Lo) <= 1e-9 * abs(Lo)
    gt, ge, gs = d.backward()
    h = 1e-7
    fe = (oracle_loss(orc, pos, vel, tab, 1.0 + h, 1.0, steps, window, bins)
          - oracle_loss(orc, pos, vel, tab, 1.0 - h, 1.0, steps, window, bins)) / (2 * h)
    fs = (oracle_loss(orc, pos, vel, tab, 1.0, 1.0 + h, steps, window, bins)
          - oracle_loss(orc, pos, vel, tab, 1.0, 1.0 - h, steps, window, bins)) / (2 * h)
    print("d/deps adjoint", ge, "oracle FD", fe, "; d/dsigma adjoint", gs, "oracle FD", fs)
    assert abs(fe - ge) <= 1e-6 * abs(fe), (fe, ge)
    assert abs(fs - gs) <= 1e-6 * abs(fs), (fs, gs)


def test_mixed_form_gradient_close_to_fp64(M):
    a, _, _ = system(M)
    b, _, _ = system(M, precision=M.PREC_MIXED)
    tab = table_of(a, seed=2, scale=0.3)
    la, lb = a.forward(tab, 1.0, 1.0), b.forward(tab, 1.0, 1.0)
    assert abs(la - lb) <= 1e-6 * abs(la)
    ga, gb = a.backward(), b.backward()
    np.testing.assert_allclose(gb[0], ga[0], rtol=1e-4, atol=1e-6 * np.abs(ga[0]).max())
    assert abs(gb[1] - ga[1]) <= 1e-4 * abs(ga[1])
    assert abs(gb[2] - ga[2]) <= 1e-4 * abs(ga[2])


def test_torch_function_and_gradient_descent(M):
    torch = pytest.importorskip("torch")
    from mrmd_gb300.torch_adjoint import trajectory_loss

    d, _, _ = system(M)
    table = torch.zeros(d.num_bins, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    loss = trajectory_loss(d, table, eps, sig)
    loss.backward()
    gt, ge, gs = d.backward()
    np.testing.assert_allclose(table.grad.numpy(), gt, rtol=1e-12)
    assert abs(float(eps.grad) - ge) <= 1e-12 * abs(ge)
    # a small gradient step on the table lowers the loss
    lr = 0.1 * float(loss) / max(float((table.grad ** 2).sum()), 1e-300)
    with torch.no_grad():
        new = table - lr * table.grad
    assert d.forward(new.numpy(), 1.0, 1.0) < float(loss)


def test_mixed_trajectory_gradient_matches_finite_differences(M):
    """The mixed form's adjoint (pairs beyond 1.4 sigma in FP32) against
    central differences of the mixed form's own loss."""
    d, pos, vel = system(M, precision=M.PREC_MIXED)
    tab = table_of(d, seed=2, scale=0.3)
    L0 = d.forward(tab, 1.0, 1.0)
    gt, ge, gs = d.backward()
    h = 1e-6
    floor = 1e-15 * abs(L0) / h * 10
    fe = central_fd(lambda e: d.forward(tab, e, 1.0), 1.0, h)
    fs = central_fd(lambda s: d.forward(tab, 1.0, s), 1.0, h)
    assert abs(fe - ge) <= 1e-5 * abs(fe) + floor, (fe, ge)
    assert abs(fs - gs) <= 1e-5 * abs(fs) + floor, (fs, gs)


def test_tf_fit_gradient_descent_next_to_iterative_update(M, tmp_path):
    """Fitting the thermodynamic-force table (mrmd_gb300.tf_fit): the
    reference's iterative update runs on exactly the trajectory the loss
    scores (the batched engine reproduces the DiffSystem forward bitwise) and
    changes the table; gradient descent on the adjoint's gradient lowers the
    loss in every iteration it takes."""
    from mrmd_gb300.tf_fit import ThermoForceFit

    n = 2000
    pos, vel = random_system(n, BOX, 3)
    rep = M.Replica(n, [0, 0, 0], BOX, [BOX[0] / 2, BOX[1] / 2, BOX[2] / 2], AT, P["seed"])
    fit = ThermoForceFit(rep, pos, vel, HY, steps=20, window=10, checkpoint_interval=5, loss_bins=32,
                         loss_sigma=1.0, capping_distance=P["cap"], rebuild_interval=5, tf_sigma=1.0, tf_range=1.0)
    t0 = np.zeros(fit.num_bins)
    L0 = fit.loss(t0)
    pd, _ = fit.diff.state()
    t1, pb = fit.update(t0)
    assert np.array_equal(pb, pd)
    assert np.all(np.isfinite(t1)) and np.abs(t1).max() > 0.0
    # the loss is summed with FP64 atomics: equal to rounding between runs
    same = lambda a, b: abs(a - b) <= 1e-12 * abs(b)
    tu, lu = fit.iterative_update(t0, 2)
    assert same(lu[0], L0) and len(lu) == 3 and np.array_equal(fit.update(t0)[0], t1)
    tg, lg = fit.gradient_descent(t0, 3)
    assert same(lg[0], L0) and len(lg) == 4
    assert all(b <= a * (1 + 1e-12) for a, b in zip(lg, lg[1:])) and lg[-1] < 0.999 * L0
    assert same(fit.loss(tg), lg[-1])
    # the fitted table round-trips through the reference's text format
    from mrmd_gb300 import io

    path = tmp_path / "tf.txt"
    io.write_table(path, fit.grid(), tg, 0)
    grid, force, bw = io.read_table(path)
    assert force.shape == (fit.num_bins, 1) and abs(bw - BOX[0] / fit.num_bins) < 1e-5
    np.testing.assert_allclose(force[:, 0], tg, rtol=1e-5, atol=1e-6 * np.abs(tg).max())
    fit.close()
