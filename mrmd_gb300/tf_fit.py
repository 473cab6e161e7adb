"""Fitting the thermodynamic-force table of one AdResS system so that the
density of its trajectory is flat, in two ways scored by the same loss:

- gradient descent on dLoss/dtable from the hand-written adjoint
  (``DiffSystem``), with a step length that halves until the loss decreases;
- the reference's iterative update (ThermodynamicForce::update,
  ThermodynamicForce.hpp:124-152: sampled density, Gaussian smoothing, its
  gradient times modulation / target density added to the table), applied by
  the batched engine at the end of the same trajectory.

The loss is the DiffSystem's: sum_b (rho_b - rho_uniform)^2 of the
Gaussian-smoothed x-density averaged over the last ``window`` steps of a
``steps``-step trajectory from a fixed initial state with seeded noise, so it
is a deterministic function of the table.  Everything runs on the GPU; this
module only sequences the calls.
"""
from __future__ import annotations

import numpy as np

from . import PREC_FP64, BatchSystem, Context, DiffSystem, default_context


class ThermoForceFit:
    """One AdResS system (single-site molecules, one replica) and its
    trajectory loss as a function of the thermodynamic-force table."""

    def __init__(self, replica, pos, vel, hybrid_diameter, steps=500, window=100, checkpoint_interval=25,
                 loss_bins=128, loss_sigma=1.0, tf_bin_width=1.2, tf_target_density=0.5, tf_modulation=1.0,
                 tf_sigma=2.4, tf_range=3.0, nu=1, rc=2.5, skin=0.3, capping_distance=0.0, shifted=True,
                 precision=PREC_FP64, dt=0.005, gamma=1.0, temperature=1.0, rebuild_interval=5,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.replica = replica
        self.pos = np.array(pos, dtype=np.float64)
        self.vel = np.array(vel, dtype=np.float64)
        self.steps = int(steps)
        physics = dict(nu=nu, rc=rc, skin=skin, capping_distance=capping_distance, shifted=shifted,
                       precision=precision, dt=dt, gamma=gamma, temperature=temperature,
                       rebuild_interval=rebuild_interval)
        self.diff = DiffSystem(replica, self.pos, self.vel, hybrid_diameter, steps=steps, window=window,
                               checkpoint_interval=checkpoint_interval, loss_bins=loss_bins, loss_sigma=loss_sigma,
                               tf_bin_width=tf_bin_width, ctx=self.ctx, **physics)
        self.num_bins = self.diff.num_bins
        # the batched engine on the same trajectory: same replica (noise
        # seed), slot order, rebuild interval and frozen compensation, with
        # the density sampled every step and one table update at its end
        self._batch_args = dict(hybrid_diameter=hybrid_diameter, tf=True, tf_bin_width=tf_bin_width,
                                tf_target_density=tf_target_density, tf_modulation=tf_modulation,
                                tf_sigma=tf_sigma, tf_range=tf_range, tf_sample_interval=1,
                                tf_update_interval=self.steps, comp_frozen=True, threads_per_row=1,
                                block_size=128, sort_every=0, graph_steps=0, list_layout=0, **physics)

    def grid(self):
        """Bin centres of the table, min + (i + 0.5) (max - min) / numBins
        along x (MultiHistogram's createGrid), as io.write_table wants them."""
        lo, hi = self.replica.box_min[0], self.replica.box_max[0]
        return lo + (np.arange(self.num_bins) + 0.5) * ((hi - lo) / self.num_bins)

    def loss(self, table):
        """Loss of the trajectory with this table (LJ epsilon = sigma = 1)."""
        return self.diff.forward(np.asarray(table, dtype=np.float64), 1.0, 1.0)

    def gradient(self, table):
        """(loss, dLoss/dtable) of the trajectory with this table."""
        L = self.loss(table)
        g, _, _ = self.diff.backward()
        return L, g

    def update(self, table):
        """The reference's update of the table after one trajectory with it:
        returns (new table, batch end state positions)."""
        b = BatchSystem([self.replica], self.pos, self.vel, ctx=self.ctx, **self._batch_args)
        try:
            b.set_thermodynamic_force([np.asarray(table, dtype=np.float64)])
            b.run(self.steps, energies=False)
            tables, _ = b.thermodynamic_force()
            p, _, _ = b.state()
            return tables[0].copy(), p
        finally:
            b.close()

    def gradient_descent(self, table, iterations, step=0.5, max_halvings=4):
        """table <- table - lr g with lr = step * L / |g|^2 (the step that
        removes the fraction `step` of L if L were linear in the table),
        halved while the loss does not decrease.  Returns (table, losses):
        losses[k] is the loss before iteration k, losses[-1] the final one."""
        t = np.array(table, dtype=np.float64)
        L, g = self.gradient(t)
        losses = [L]
        for _ in range(int(iterations)):
            gg = float(g @ g)
            if gg == 0.0:
                losses.append(L)
                continue
            lr = step * L / gg
            for _ in range(max_halvings + 1):
                cand = t - lr * g
                Lc = self.loss(cand)
                if Lc < L:
                    break
                lr *= 0.5
            if Lc < L:
                t = cand
                L, g = self.gradient(t)
            losses.append(L)
        return t, losses

    def iterative_update(self, table, iterations):
        """table <- update(table), `iterations` times.  Returns (table,
        losses) as gradient_descent does."""
        t = np.array(table, dtype=np.float64)
        losses = [self.loss(t)]
        for _ in range(int(iterations)):
            t, _ = self.update(t)
            losses.append(self.loss(t))
        return t, losses

    def close(self):
        self.diff.close()
