"""The AdResS step composed from the oracle's actions, in the order of the
fused steppers (Langevin pre; every K steps UpdateMolecules, MultiRes
exchange, ghosts and the molecule half list, else the ghost update;
UpdateMolecules; forces = 0; LJ_IdealGas::run; ContributeMoleculeForceToAtoms;
ThermodynamicForce::apply; ghost fold-back; VV post; TF sample / update).
Test infrastructure only: it drives the oracle, the checker."""
import numpy as np


def random_system(n, box, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 1, (n, 3)) * np.asarray(box)
    vel = rng.normal(0, 1, (n, 3))
    return pos, vel


def oracle_loop(orc, pos, vel, box, nsteps, p, slab_center=None, seed=None, box_min=(0.0, 0.0, 0.0),
                tf_table=None, comp_frozen=False, on_step=None, tf_out=None):
    """Returns positions, velocities, per-step energies, the TF table and the
    LJ_IdealGas mean compensation energies after nsteps.  tf_table sets the
    initial thermodynamic-force table; comp_frozen starts LJ_IdealGas at run 1
    so that its compensation means stay zero; on_step(st, positions) sees the
    positions after every step; tf_out (a dict) receives the density profile
    accumulated since the last update and its sample count."""
    n = len(pos)
    lo = np.asarray(box_min, dtype=np.float64)
    hi = lo + np.asarray(box, dtype=np.float64)
    rlist = p["rc"] + p["skin"]
    sd = orc.subdomain(list(lo), list(hi), rlist)
    a = orc.Atoms.from_positions(pos, capacity=8 * n + 64)
    a.vel[:n] = vel
    m = orc.Molecules(8 * n + 64)
    m.atomsOffset[:n] = np.arange(n)
    m.numAtoms[:n] = 1
    m.numLocal = n
    center = slab_center if slab_center is not None else list((lo + hi) / 2)
    slab = orc.slab(center, p["at"], p["hy"], p["nu"])
    ljig = orc.LJIdealGas(p["cap"], p["rc"], p["sigma"], p["epsilon"], True)
    if comp_frozen:
        ljig.s.runCounter = 1
    tf = orc.ThermodynamicForce([p["rho"]], sd, p["binw"], [p["mod"]], False, True)
    if tf_table is not None:
        tf.force[:, 0] = tf_table
    energies = []
    corr = co = no = None
    sd_seed = p["seed"] if seed is None else seed
    for st in range(nsteps):
        orc.langevin_pre(a, p["dt"], p["gamma"], p["T"], sd_seed, st)
        if st % p["K"] == 0:
            a.numGhost = 0
            m.numGhost = 0
            orc.update_molecules(m, a, slab)
            orc.multires_map_into_domain(sd, m, a)
            corr = orc.multires_create_ghosts(m, a, sd)
            co, no = orc.build_half_list(m.pos, m.numLocal + m.numGhost, 0, m.numLocal, rlist,
                                         sd.minGhostCorner, sd.maxGhostCorner, 1.0, 160)
        else:
            orc.update_ghosts(a, corr, sd)
        orc.update_molecules(m, a, slab)
        a.force[:] = 0
        m.force[:] = 0
        energies.append(ljig.run(m, co, no, a))
        orc.contribute_molecule_force(m, a)
        tf.apply(a)
        orc.ghost_to_real(a, corr)
        orc.vv_post(a, p["dt"])
        if st % p["S"] == 0:
            tf.sample(a)
        if (st + 1) % p["U"] == 0:
            tf.update(p["tfs"], p["tfr"])
        if on_step is not None:
            on_step(st, a.pos[:n])
    if tf_out is not None:
        tf_out["density"] = tf.density[:, 0].copy()
        tf_out["samples"] = tf.samples
    return (a.pos[:n].copy(), a.vel[:n].copy(), np.array(energies), tf.force[:, 0].copy(),
            ljig.mean[:, 0].copy())
