"""Host logic of the thermodynamic-force table fit (mrmd_gb300.tf_fit) with
the GPU trajectory replaced by a fake quadratic loss: the step length of the
gradient descent, monotone losses, the sequencing of the iterative update,
and the bin centres."""
import numpy as np


class FakeDiff:
    """L(t) = |A t - b|^2, dL/dt = 2 A^T (A t - b); forward/backward as
    DiffSystem's (backward returns the gradient of the last forward)."""

    def __init__(self, n, seed=0):
        rng = np.random.default_rng(seed)
        self.A = rng.normal(size=(n + 3, n)) / np.sqrt(n)
        self.b = rng.normal(size=n + 3)
        self.calls = 0

    def forward(self, table, eps, sig):
        self.t = np.array(table, dtype=np.float64)
        self.calls += 1
        r = self.A @ self.t - self.b
        return float(r @ r)

    def backward(self):
        return 2.0 * self.A.T @ (self.A @ self.t - self.b), 0.0, 0.0


class FakeReplica:
    box_min = (2.0, 0.0, 0.0)
    box_max = (10.0, 5.0, 5.0)


def fit_with(diff, n):
    from mrmd_gb300.tf_fit import ThermoForceFit

    fit = object.__new__(ThermoForceFit)
    fit.diff = diff
    fit.num_bins = n
    fit.replica = FakeReplica()
    return fit


def test_gradient_descent_lowers_the_loss_every_iteration():
    n = 12
    d = FakeDiff(n)
    fit = fit_with(d, n)
    t, losses = fit.gradient_descent(np.zeros(n), 15)
    assert len(losses) == 16
    assert all(b <= a for a, b in zip(losses, losses[1:]))
    assert losses[-1] < 0.5 * losses[0]
    # the returned table is the one the last loss belongs to
    assert abs(d.forward(t, 1.0, 1.0) - losses[-1]) <= 1e-12 * losses[-1]


def test_gradient_descent_keeps_the_table_when_no_step_helps():
    """At a minimum (zero gradient) nothing moves and the loss repeats."""
    n = 6
    d = FakeDiff(n, seed=3)
    t_star = np.linalg.lstsq(d.A, d.b, rcond=None)[0]
    fit = fit_with(d, n)
    t, losses = fit.gradient_descent(t_star, 3)
    np.testing.assert_allclose(t, t_star, rtol=0, atol=1e-9)
    assert max(losses) - min(losses) <= 1e-9 * max(losses[0], 1.0)


def test_iterative_update_sequencing():
    n = 8
    d = FakeDiff(n, seed=5)
    fit = fit_with(d, n)
    seen = []

    def update(t):
        seen.append(np.array(t))
        return t - 0.1 * (2.0 * d.A.T @ (d.A @ t - d.b)), None

    fit.update = update
    t, losses = fit.iterative_update(np.zeros(n), 4)
    assert len(losses) == 5 and len(seen) == 4
    np.testing.assert_array_equal(seen[0], np.zeros(n))
    assert abs(losses[-1] - d.forward(t, 1.0, 1.0)) <= 1e-12 * losses[-1]


def test_grid_is_the_bin_centres():
    fit = fit_with(FakeDiff(4), 4)
    np.testing.assert_allclose(fit.grid(), [3.0, 5.0, 7.0, 9.0], rtol=0, atol=1e-15)
