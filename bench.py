"""Benchmark: atom-steps/s of the LJ NVE hot path on one GB300.

Workload: 4,000,000-atom LJ fluid (fcc 100^3 cells, reduced density 0.8442,
T* = 0.728 Maxwell-Boltzmann velocities from a seed, rc = 2.5 sigma shifted,
skin 0.3 sigma, half/full Verlet list rebuilt every 10 steps, dt = 0.005),
run in the plain FP64 form and in the mixed form.  `value` is the mixed
form's atom-steps/s with the state resident in HBM; the FP64 form, the force
error of the mixed form against FP64 on identical positions and the NVE
drift of both are reported beside it.  `e2e` runs the same workload through
the public stepper API from pinned host buffers (state upload, per-step
energy read-back, final state download inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

Under torchrun (N > 1) every rank runs an independent replica (replicas
only: the hot path has no exchange step) and rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s"
WORKLOAD = ("LJ fluid 4,000,000 atoms (fcc 100^3, rho 0.8442, T 0.728, rc 2.5 shifted, skin 0.3, rebuild/10, "
            "dt 0.005; atoms re-sorted every 4th rebuild)")


def fcc(cells, rho=0.8442):
    a = (4.0 / rho) ** (1.0 / 3.0)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(cells)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = ((g[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25) * a
    return pos, a * cells


def mb_velocities(n, T, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(0.0, np.sqrt(T), (n, 3))
    v -= v.mean(0)
    return v


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def issue_roofline(torch, device, per_atom, n, kern_ms, clocks):
    """The pair kernel against the GPU's instruction issue rate (one warp
    instruction per scheduler and clock, 4 schedulers per SM): thread
    instructions per atom from the ncu summary x atoms / kernel time, against
    SMs x 4 x 32 lanes x the SM clock sampled during the timed run."""
    if per_atom is None or not clocks or not clocks.get("sm_mhz"):
        return None
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    peak = sms * 4 * 32 * clocks["sm_mhz"] * 1e6
    achieved = per_atom * n / (kern_ms * 1e-3)
    return {"unit": "thread instructions/s", "thread_instructions_per_atom": per_atom, "achieved": achieved,
            "peak": peak, "frac": achieved / peak, "sms": sms, "sm_mhz": clocks["sm_mhz"]}


def load_traffic(kernel, key="dram_bytes_per_atom"):
    """A per-atom figure of one pair-kernel launch (DRAM bytes, thread
    instructions) from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.lstrip().startswith("#"):
                continue
            parts = dict(kv.split("=", 1) for kv in line.split() if "=" in kv)
            if parts.get("kernel") == kernel and key in parts:
                return float(parts[key])
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms in the
    background.  The sampler is running (its first line written) before the
    `with` body starts; time_run() marks the timed window and summary() keeps
    the samples inside it (the nearest one when the window is shorter than
    the sampling interval)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None
        self.window = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return None
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(c[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    rows.append((ts, float(c[2]), float(c[3]),
                                 {n for n, v in zip(names, c[6:10]) if v.lower().startswith("active")}))
                except ValueError:
                    continue
        os.unlink(self.path)
        if not rows:
            return None
        inside = rows
        if self.window is not None:
            t0, t1 = self.window
            inside = [r for r in rows if t0 <= r[0] <= t1]
            if not inside:
                inside = [min(rows, key=lambda r: abs(r[0] - 0.5 * (t0 + t1)))]
        reasons = set().union(*(r[3] for r in inside))
        return {"sm_mhz": float(np.median([r[1] for r in inside])), "sm_max_mhz": float(max(r[2] for r in inside)),
                "samples": len(inside), "reasons": sorted(reasons)}


def run_cpu(pos, vel, L, steps, warmup, budget_s, threads):
    """The oracle (CPU restatement of the reference loop, OpenMP) on the same
    workload: examples/02_LennardJones_NVE.cpp:135-216 with rebuild every 10."""
    from oracle import oracle as O

    O.set_threads(threads)
    rc, skin, dt, K = 2.5, 0.3, 0.005, 10
    n = len(pos)
    sd = O.subdomain([0, 0, 0], [L] * 3, rc + skin)
    a = O.Atoms.from_positions(pos, capacity=int(n * 1.3) + 1024)
    a.vel[:n] = vel
    tab = O.lj_table(0.0, rc, 1.0, 1.0, 1, True)
    state = {}

    def rebuild():
        a.numGhost = 0
        O.map_into_domain(a, sd)
        state["corr"] = O.create_ghosts(a, sd)
        state["list"] = O.build_half_list(a.pos, a.n, 0, a.numLocal, rc + skin, sd.minGhostCorner,
                                          sd.maxGhostCorner, 1.0, 64)

    def forces():
        a.force[: a.n] = 0.0
        co, no = state["list"]
        E, W = O.lj_apply(tab, rc * rc, a, co, no)
        O.ghost_to_real(a, state["corr"])
        return E

    rebuild()
    forces()

    def step(s):
        O.vv_pre(a, dt)
        if s % K == 0:
            rebuild()
        else:
            O.update_ghosts(a, state["corr"], sd)
        forces()
        O.vv_post(a, dt)

    t0 = time.perf_counter()
    s = 0
    while s < warmup and time.perf_counter() - t0 < budget_s / 4:
        step(s)
        s += 1
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        step(s)
        s += 1
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dtime = time.perf_counter() - t0
    return n * done / dtime, done, dtime


def cpu_info():
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                model = line.split(":", 1)[1].strip()
    except OSError:
        pass
    return os.cpu_count() or 1, model


def reference_arm(args, rank, world):
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    cells = args.cells
    pos, L = fcc(cells)
    vel = mb_velocities(len(pos), 0.728, 0)
    ncores, model = cpu_info()
    value, done, dtime = run_cpu(pos, vel, L, args.steps, args.warmup, args.cpu_budget, ncores)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * dtime / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded fcc lattice + Maxwell-Boltzmann velocities)",
        "config": {"workload": WORKLOAD, "atoms": len(pos), "form": "FP64 half list, OpenMP atomics",
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": ncores, "kind": "port",
                         "sample": f"{done} steps of the {len(pos)}-atom system on {ncores} threads ({model}); "
                                   "CPU restatement of the reference (Kokkos/Cabana not buildable here)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(value, dist, device):
    """The slowest rank's time: every rank's replica must be done before the job is."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, steps, world, seconds):
    """Whole-job throughput of independent replicas (one per rank): all units
    of all ranks over the slowest rank's time."""
    return units_per_rank * steps * world / seconds


def time_run(torch, M, sysm, steps, stream, clk=None):
    """CUDA-event time of `steps` steps on the stepper's stream (ms), wall
    time (s), energies and kernel launches; clk (a running ClockSampler)
    gets the timed window."""
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sysm.ctx.sync()
    l0 = sysm.ctx.launches
    w0 = time.time()
    t0 = time.perf_counter()
    ev0.record(stream)
    e = sysm.run(steps)
    ev1.record(stream)
    ev1.synchronize()
    wall = time.perf_counter() - t0
    if clk is not None:
        clk.mark(w0, time.time())
    return ev0.elapsed_time(ev1), wall, e, sysm.ctx.launches - l0


DRIFT_SETUP = ("32,000 atoms (fcc 20^3, same density, T 0.728 start), 2,000 FP64 steps to equilibrate, then "
               "200,000 steps (1000 tau) per form from that state, for 3 velocity seeds (mean and sd reported); "
               "drift = slope of a least-squares line through (E_pot + E_kin)/N of every step, both summed on "
               "the device inside the step")
MIXED_DTYPE = ("f64 state; pair arithmetic f32 beyond 1.5 sigma, double-float closer; energy/virial sums "
               "double-float")


DRIFT_SEEDS = (7, 8, 9)


def nve_drift(M, ctx, forms, cells=20, equil=2000, steps=200000, dt=0.005, seeds=DRIFT_SEEDS):
    """Energy drift per atom per 1000 tau of each form, from the per-step
    records of the observing stepper (no host transfer inside the run), for
    each seed of the initial velocities: mean, standard deviation and the
    per-seed values."""
    pos, L = fcc(cells)
    per = {f: [] for f in forms}
    fluct = {f: [] for f in forms}
    mom = {f: [] for f in forms}
    for seed in seeds:
        vel = mb_velocities(len(pos), 0.728, seed)
        eq = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=M.PREC_FP64, ctx=ctx)
        eq.run(equil, energies=False)
        p, v, _ = eq.state()
        eq.close()
        for form in forms:
            prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
            s = M.LJSystem(p, v, [0, 0, 0], [L] * 3, precision=prec, observe=True, ctx=ctx)
            rec = s.run_observed(steps)
            s.close()
            et = (rec[:, 0] + rec[:, 2]) / len(p)
            t = np.arange(steps) * dt
            per[form].append(float(np.polyfit(t, et, 1)[0]) * 1000.0)
            fluct[form].append(float(et.std()))
            # largest component of the velocity sum (the reference's
            # getSystemMomentum) reached during the run, per atom
            mom[form].append(float(np.abs(rec[:, 3:6]).max()) / len(p))
    return {f: dict(drift=float(np.mean(per[f])), drift_sd=float(np.std(per[f], ddof=1)) if len(per[f]) > 1 else None,
                    drift_per_seed=per[f], fluct=float(np.mean(fluct[f])), momentum_max=float(np.max(mom[f])))
            for f in forms}


def adress_leg(M, ctx, torch, stream, molecules, forms, warmup=300, steps=100):
    """The AdResS workload (scaled to `molecules` at density 0.5) through the
    drop-in stepper (AdResSSystem, mrmd_adress_*: the batched engine with one
    replica for these unit-mass molecules), both forms: ms per step,
    atom-steps/s and the force error of the mixed form against FP64 on the
    first step's identical positions."""
    c = adress_config(molecules)
    pos, vel = adress_initial(100, c)
    n = len(pos)
    out, forces = {}, {}
    for form in forms:
        prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
        b = M.AdResSSystem(pos, vel, [0, 0, 0], list(c["box"]), list(c["center"]), c["at"], c["hy"], c["nu"],
                           rc=c["rc"], skin=c["skin"], capping_distance=c["cap"], precision=prec, dt=c["dt"],
                           rebuild_interval=c["K"], gamma=c["gamma"], temperature=c["T"], seed=1234, tf=True,
                           tf_bin_width=c["binw"], tf_target_density=c["rho"], tf_modulation=c["mod"],
                           tf_sigma=c["tfs"], tf_range=c["tfr"], tf_sample_interval=c["S"],
                           tf_update_interval=c["U"], ctx=ctx)
        b.run(1, energies=False)
        forces[form] = b.state()[2]
        # the random start relaxes over the first few hundred steps; its list
        # rows grow meanwhile (capacity recoveries replay whole graphs)
        b.run(warmup - 1, energies=False)
        ms, wall, e, launches = time_run(torch, M, b, steps, stream)
        out[form] = {"ms_per_step": ms / steps, "atom_steps_per_s": n * steps / (ms * 1e-3)}
        b.close()
    res = {"molecules": n, "forms": out, "warmup_steps": warmup, "timed_steps": steps,
           "engine": ("AdResSSystem (mrmd_adress_*): batched engine with one replica, CUDA graphs of 50 steps"
                      + (", the steps between rebuilds as one persistent launch" if n >= 1000000 else ""))}
    if {"fp64", "mixed"} <= out.keys():
        res["mixed_over_fp64"] = out["mixed"]["atom_steps_per_s"] / out["fp64"]["atom_steps_per_s"]
        fa, fb = forces["fp64"], forces["mixed"]
        d = np.linalg.norm(fa - fb, axis=1)
        mag = np.linalg.norm(fa, axis=1)
        rms = float(np.sqrt((mag ** 2).mean()))
        res["force_error_mixed_vs_fp64"] = {"max_abs_over_rms": float(d.max() / rms),
                                            "max_relative_floor_0.1rms": float((d / np.maximum(mag, 0.1 * rms)).max())}
    return res


def time_pair_kernel(torch, sysm, stream, reps=20):
    sysm.eval_forces()
    for _ in range(3):
        sysm.launch_pair_kernel()
    sysm.ctx.sync()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        sysm.launch_pair_kernel()
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1) / reps


ADRESS = dict(n=34560, box=(120.0, 24.0, 24.0), center=(60.0, 12.0, 12.0), at=30.0, hy=10.0, nu=1, rc=2.5,
              skin=0.3, cap=0.78420, gamma=1.0, T=1.0, binw=1.2, rho=0.5, mod=1.0, tfs=2.4, tfr=3.0, S=1,
              U=1000, dt=0.005, K=10)
ADRESS_WORKLOAD = ("AdResS LJ<->ideal gas, 34,560 single-site molecules in 120x24x24, atomistic slab 30, hybrid 10, "
                   "cos^2, rc 2.5 with force cap 1000 (r_cap 0.7842), Langevin T=1 gamma=1, thermodynamic force "
                   "100 bins sampled every step / updated every 1000, rebuild/10, dt 0.005")


def adress_config(molecules=None):
    """The AdResS workload, or the same physics at `molecules` molecules: the
    box, slab centre and atomistic width scaled by the same factor (density
    0.5 kept), hybrid width and bin width unchanged."""
    c = dict(ADRESS)
    if molecules and molecules != c["n"]:
        f = (molecules / c["n"]) ** (1.0 / 3.0)
        c.update(n=int(molecules), box=tuple(x * f for x in c["box"]), center=tuple(x * f for x in c["center"]),
                 at=c["at"] * f)
    return c


def adress_initial(seed=0, c=None):
    c = c or ADRESS
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, 1.0, (c["n"], 3)) * np.asarray(c["box"])
    vel = mb_velocities(c["n"], c["T"], seed + 1)
    return pos, vel


def run_adress_cpu(pos, vel, steps, warmup, budget_s, threads, geometry=None):
    """Oracle loop of the AdResS step (the composition in mrmd_gb300/csrc/adress_md.cu).
    geometry overrides box, center, at and hy of the AdResS workload."""
    from oracle import oracle as O

    O.set_threads(threads)
    c = dict(ADRESS, **(geometry or {}))
    n = len(pos)
    rlist = c["rc"] + c["skin"]
    sd = O.subdomain([0, 0, 0], list(c["box"]), rlist)
    a = O.Atoms.from_positions(pos, capacity=8 * n + 64)
    a.vel[:n] = vel
    m = O.Molecules(8 * n + 64)
    m.atomsOffset[:n] = np.arange(n)
    m.numAtoms[:n] = 1
    m.numLocal = n
    slab = O.slab(list(c["center"]), c["at"], c["hy"], c["nu"])
    ljig = O.LJIdealGas(c["cap"], c["rc"], 1.0, 1.0, True)
    tf = O.ThermodynamicForce([c["rho"]], sd, c["binw"], [c["mod"]], False, True)
    st = {"corr": None, "list": None}

    def step(s):
        O.langevin_pre(a, c["dt"], c["gamma"], c["T"], 1234, s)
        if s % c["K"] == 0:
            a.numGhost = 0
            m.numGhost = 0
            O.update_molecules(m, a, slab)
            O.multires_map_into_domain(sd, m, a)
            st["corr"] = O.multires_create_ghosts(m, a, sd)
            st["list"] = O.build_half_list(m.pos, m.numLocal + m.numGhost, 0, m.numLocal, rlist,
                                           sd.minGhostCorner, sd.maxGhostCorner, 1.0, 96)
        else:
            O.update_ghosts(a, st["corr"], sd)
        O.update_molecules(m, a, slab)
        a.force[: a.n] = 0.0
        m.force[: m.numLocal + m.numGhost] = 0.0
        ljig.run(m, st["list"][0], st["list"][1], a)
        O.contribute_molecule_force(m, a)
        tf.apply(a)
        O.ghost_to_real(a, st["corr"])
        O.vv_post(a, c["dt"])
        if s % c["S"] == 0:
            tf.sample(a)
        if (s + 1) % c["U"] == 0:
            tf.update(c["tfs"], c["tfr"])

    s = 0
    for _ in range(warmup):
        step(s)
        s += 1
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        step(s)
        s += 1
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dtime = time.perf_counter() - t0
    return n * done / dtime, done, dtime


def adress_main(args, rank, world, local_rank):
    """Config-2 AdResS step, FP64 and mixed forms (a separate measurement line)."""
    import torch

    import mrmd_gb300 as M

    torch.cuda.set_device(local_rank)
    ctx = M.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    c = adress_config(args.molecules)
    pos, vel = adress_initial(100 + rank, c)
    n = len(pos)
    workload = ADRESS_WORKLOAD if n == ADRESS["n"] else (
        f"{ADRESS_WORKLOAD}; scaled to {n:,} molecules in {c['box'][0]:.1f}x{c['box'][1]:.1f}x{c['box'][2]:.1f}, "
        f"atomistic slab {c['at']:.1f}")
    res = {}
    forces = {}
    for form in [f.strip() for f in args.forms.split(",") if f.strip()]:
        prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
        s = M.AdResSSystem(pos, vel, [0, 0, 0], list(c["box"]), list(c["center"]), c["at"], c["hy"], c["nu"],
                           rc=c["rc"], skin=c["skin"], capping_distance=c["cap"], precision=prec, dt=c["dt"],
                           rebuild_interval=c["K"], gamma=c["gamma"], temperature=c["T"], tf=True,
                           tf_bin_width=c["binw"], tf_target_density=c["rho"], tf_modulation=c["mod"],
                           tf_sigma=c["tfs"], tf_range=c["tfr"], tf_sample_interval=c["S"],
                           tf_update_interval=c["U"], ctx=ctx)
        s.run(args.warmup)
        with ClockSampler(local_rank) as clk:
            ms, wall, e, launches = time_run(torch, M, s, args.steps, stream, clk)
        res[form] = dict(ms=ms, value=n * args.steps / (ms * 1e-3), launches=launches, clocks=clk.summary(),
                         stats=s.stats())
        s.close()
        # the same system on the batched engine (one replica): four launches per step, 50-step graphs
        rep = M.Replica(n, [0, 0, 0], list(c["box"]), list(c["center"]), c["at"], 1234)
        b = M.BatchSystem([rep], pos, vel, hybrid_diameter=c["hy"], nu=c["nu"], rc=c["rc"], skin=c["skin"],
                          capping_distance=c["cap"], precision=prec, dt=c["dt"], gamma=c["gamma"],
                          temperature=c["T"], tf=True, tf_bin_width=c["binw"], tf_target_density=c["rho"],
                          tf_modulation=c["mod"], tf_sigma=c["tfs"], tf_range=c["tfr"], tf_sample_interval=c["S"],
                          tf_update_interval=c["U"], rebuild_interval=c["K"], sort_every=5, graph_steps=50, ctx=ctx)
        # the first step's forces act on identical positions in both forms (the
        # pre-force integration is FP64 in both)
        b.run(1, energies=False)
        forces[form] = b.state()[2]
        b.run(max(args.warmup, 50) - 1, energies=False)
        with ClockSampler(local_rank) as clk:
            ms, wall, e, launches = time_run(torch, M, b, args.steps, stream, clk)
        st = b.stats()
        res[form + "_batch_engine"] = dict(ms=ms, value=n * args.steps / (ms * 1e-3), launches=launches,
                                           clocks=clk.summary(), stats={"pairs": st["pairs"],
                                                                        "ghost_molecules": st["ghost_molecules"]})
        b.close()
    ferr = None
    if "fp64" in forces and "mixed" in forces:
        fa, fb = forces["fp64"], forces["mixed"]
        d = np.linalg.norm(fa - fb, axis=1)
        mag = np.linalg.norm(fa, axis=1)
        rms = float(np.sqrt((mag ** 2).mean()))
        ferr = {"max_abs_over_rms": float(d.max() / rms),
                "max_relative_floor_0.1rms": float((d / np.maximum(mag, 0.1 * rms)).max())}
    cpu = None
    if not args.no_cpu:
        ncores, model = cpu_info()
        geom = {k: c[k] for k in ("box", "center", "at")}
        cv, done, ctime = run_adress_cpu(pos, vel, 10 ** 6, 3, args.cpu_budget, ncores, geom)
        cpu = {"value": cv, "unit": METRIC, "cores": ncores, "kind": "port",
               "sample": f"{done} steps of the {n}-molecule system, {ncores} OpenMP threads ({model})"}
    head = max(res, key=lambda f: res[f]["value"])
    r = res[head]
    print(json.dumps({
        "metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if head.startswith("fp64") else "f64 state, f32 double-float pair arithmetic",
        "data": "synthetic (seeded uniform positions, Maxwell-Boltzmann velocities)",
        "config": {"workload": workload, "molecules": n, "form": head,
                   "forms": {f: {"atom_steps_per_s": res[f]["value"], "ms_per_step": res[f]["ms"] / args.steps,
                                 "kernel_launches": res[f]["launches"], "list_pairs": res[f]["stats"]["pairs"],
                                 "ghost_molecules": res[f]["stats"]["ghost_molecules"]} for f in res},
                   "force_error_mixed_vs_fp64": ferr},
        "gpu_launches": r["launches"], "clocks": r["clocks"], "cpu_baseline": cpu}), flush=True)


BATCH = dict(replicas=512, nmin=1000, nmax=50000, cross=20.0, rho=(0.4, 0.6), at=(10.0, 30.0), hy=8.0,
             graph=50, seed=4)
BATCH_WORKLOAD = ("512 independent AdResS replicas (LJ<->ideal gas, single-site), sizes log-uniform 1,000-50,000, "
                  "cross-section 20x20, density U(0.4, 0.6), atomistic slab U(10, 30), hybrid 8, otherwise the "
                  "34,560-molecule AdResS workload's physics; one launch per phase for all replicas, CUDA graphs "
                  "of 50 steps")


def batch_replicas(M, count=None):
    """Seeded replica set: sizes, boxes, slabs and initial states."""
    b = BATCH
    rng = np.random.default_rng(b["seed"])
    R = count or b["replicas"]
    sizes = np.exp(rng.uniform(np.log(b["nmin"]), np.log(b["nmax"]), R)).astype(np.int64)
    rhos = rng.uniform(*b["rho"], R)
    ats = rng.uniform(*b["at"], R)
    reps, P_, V_, geoms = [], [], [], []
    for r in range(R):
        lx = float(sizes[r] / (b["cross"] * b["cross"] * rhos[r]))
        box = (lx, b["cross"], b["cross"])
        center = (lx / 2, b["cross"] / 2, b["cross"] / 2)
        reps.append(M.Replica(int(sizes[r]), [0, 0, 0], box, center, float(ats[r]), 10_000 + r))
        P_.append(rng.uniform(0.0, 1.0, (int(sizes[r]), 3)) * np.asarray(box))
        V_.append(rng.normal(0.0, 1.0, (int(sizes[r]), 3)))
        geoms.append(dict(box=box, center=center, at=float(ats[r]), hy=b["hy"]))
    return reps, np.concatenate(P_), np.concatenate(V_), geoms


def batch_main(args, rank, world, local_rank):
    """Config-4 batch of AdResS replicas, FP64 and mixed forms."""
    import torch

    import mrmd_gb300 as M

    torch.cuda.set_device(local_rank)
    ctx = M.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    c = ADRESS
    reps, pos, vel, geoms = batch_replicas(M, args.replicas)
    n = len(pos)
    res = {}
    forces = {}
    for form in [f.strip() for f in args.forms.split(",") if f.strip()]:
        prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
        s = M.BatchSystem(reps, pos, vel, hybrid_diameter=BATCH["hy"], nu=c["nu"], rc=c["rc"], skin=c["skin"],
                          capping_distance=c["cap"], precision=prec, dt=c["dt"], gamma=c["gamma"],
                          temperature=c["T"], tf=True, tf_bin_width=c["binw"], tf_target_density=c["rho"],
                          tf_modulation=c["mod"], tf_sigma=c["tfs"], tf_range=c["tfr"], tf_sample_interval=c["S"],
                          tf_update_interval=c["U"], threads_per_row=4 if args.list_layout == 2 else 1,
                          block_size=128, rebuild_interval=c["K"], sort_every=5, graph_steps=BATCH["graph"],
                          list_layout=args.list_layout, ctx=ctx)
        s.run(1)
        forces[form] = s.state()[2]
        s.run(BATCH["graph"] - 1)
        tuned, trials = (s.tuning, []) if args.no_autotune else s.autotune(trial_steps=BATCH["graph"])
        # the random start relaxes over the first few hundred steps; its list
        # rows grow meanwhile (capacity recoveries replay whole graphs)
        s.run(max(args.warmup, 300))
        with ClockSampler(local_rank) as clk:
            ms, wall, e, launches = time_run(torch, M, s, args.steps, stream, clk)
        res[form] = dict(ms=ms, value=n * args.steps / (ms * 1e-3), launches=launches, clocks=clk.summary(),
                         stats=s.stats(), lstats=s.list_stats(), tuning=tuned,
                         trials=[dict(t, ms_per_step=m) for t, m in trials])
        s.close()
    ferr = None
    if "fp64" in forces and "mixed" in forces:
        fa, fb = forces["fp64"], forces["mixed"]
        d = np.linalg.norm(fa - fb, axis=1)
        mag = np.linalg.norm(fa, axis=1)
        rms = float(np.sqrt((mag ** 2).mean()))
        ferr = {"max_abs_over_rms": float(d.max() / rms),
                "max_relative_floor_0.1rms": float((d / np.maximum(mag, 0.1 * rms)).max())}
    cpu = None
    if not args.no_cpu:
        ncores, model = cpu_info()
        done_total, t_total, atoms_steps = 0, 0.0, 0.0
        budget = args.cpu_budget
        for r in range(3):  # the first replicas of the set, one after another
            sl = slice(int(sum(x.num_molecules for x in reps[:r])), int(sum(x.num_molecules for x in reps[:r + 1])))
            cv, done, ctime = run_adress_cpu(pos[sl], vel[sl], 10 ** 6, 1, budget / 3, ncores, geoms[r])
            atoms_steps += cv * ctime
            t_total += ctime
            done_total += done
        cpu = {"value": atoms_steps / t_total, "unit": METRIC, "cores": ncores, "kind": "port",
               "sample": f"the first 3 replicas run one after another by the oracle loop, {done_total} steps in "
                         f"{t_total:.1f} s, {ncores} OpenMP threads ({model})"}
    head = "mixed" if "mixed" in res else next(iter(res))
    r = res[head]
    out = {
        "metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if head == "fp64" else "f64 state, f32 double-float pair arithmetic",
        "data": "synthetic (seeded replica sizes, boxes and slabs; uniform positions, normal velocities)",
        "config": {"workload": BATCH_WORKLOAD, "replicas": len(reps), "molecules": n, "form": head,
                   "forms": {f: {"atom_steps_per_s": res[f]["value"], "ms_per_step": res[f]["ms"] / args.steps,
                                 "kernel_launches": res[f]["launches"], "list_pairs": res[f]["stats"]["pairs"],
                                 "list_entries": res[f]["lstats"]["entries"],
                                 "list_lane_efficiency": res[f]["lstats"]["lane_efficiency"],
                                 "ghost_molecules": res[f]["stats"]["ghost_molecules"],
                                 "graph_launches": res[f]["stats"]["graph_launches"],
                                 "tuning": res[f]["tuning"], "autotune_trials": res[f]["trials"]}
                             for f in res}},
        "gpu_launches": r["launches"], "clocks": r["clocks"], "cpu_baseline": cpu}
    if "fp64" in res and "mixed" in res:
        out["config"]["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
        out["config"]["force_error_mixed_vs_fp64"] = ferr
    print(json.dumps(out), flush=True)


DIFF = dict(n=65536, box=(256.0, 16.0, 32.0), center=(128.0, 8.0, 16.0), at=30.0, hy=10.0, steps=500, window=100,
            ckpt=25, loss_bins=128, loss_sigma=1.0, tf_bins=100, K=5, relax=2000)
DIFF_WORKLOAD = ("AdResS trajectory gradient: 65,536 single-site molecules in 256x16x32 (density 0.5), slab 30 / hybrid "
                 "10, Langevin T=1 gamma=1 with counter-based noise, rc 2.5 with force cap 1000, relaxed for 2000 "
                 "steps from a uniform placement and ordered by cell, then 500 differentiated steps, loss = "
                 "squared deviation from uniform of the sigma_b=1 Gaussian-smoothed 128-bin x-density averaged over "
                 "the last 100 steps; gradient w.r.t. the 100 thermodynamic-force coefficients and LJ epsilon, sigma "
                 "by the hand-written adjoint with a checkpoint every 25 steps")


def diff_main(args, rank, world, local_rank):
    """Config-5 differentiation: forward + adjoint of a 500-step AdResS trajectory."""
    import torch

    import mrmd_gb300 as M

    torch.cuda.set_device(local_rank)
    ctx = M.Context(local_rank)
    c, g = ADRESS, DIFF
    rng = np.random.default_rng(5 + rank)
    n = g["n"]
    pos = rng.uniform(0.0, 1.0, (n, 3)) * np.asarray(g["box"])
    vel = mb_velocities(n, c["T"], 6 + rank)
    rep = M.Replica(n, [0, 0, 0], list(g["box"]), list(g["center"]), g["at"], 1234)
    # relax the uniform placement with the capped potential under the thermostat
    relax = M.BatchSystem([rep], pos, vel, hybrid_diameter=g["hy"], capping_distance=c["cap"], dt=c["dt"],
                          gamma=c["gamma"], temperature=c["T"], tf=False, rebuild_interval=g["K"], sort_every=0,
                          graph_steps=50, ctx=ctx)
    relax.run(g["relax"], energies=False)
    pos, vel, _ = relax.state()
    relax.close()
    # molecules in cell order (cells of the list radius, x-major): a warp's rows
    # then belong to one region of the slab (atomistic, hybrid or coarse
    # grained) instead of a random mix; the differentiation engine keeps the
    # order it is given (its Langevin noise is keyed by slot)
    edge = 2.5 + 0.3
    cells = np.floor(pos / edge).astype(np.int64)
    ncell = np.floor(np.asarray(g["box"]) / edge).astype(np.int64)
    cells = np.minimum(np.maximum(cells, 0), ncell - 1)
    key = (cells[:, 0] * ncell[1] + cells[:, 1]) * ncell[2] + cells[:, 2]
    order = np.argsort(key, kind="stable")
    pos, vel = pos[order], vel[order]
    table = np.zeros(g["tf_bins"])
    res = {}
    for form in [f.strip() for f in args.forms.split(",") if f.strip()]:
        prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
        d = M.DiffSystem(rep, pos, vel, hybrid_diameter=g["hy"], steps=g["steps"], window=g["window"],
                         checkpoint_interval=g["ckpt"], loss_bins=g["loss_bins"], loss_sigma=g["loss_sigma"],
                         capping_distance=c["cap"], precision=prec, dt=c["dt"], gamma=c["gamma"],
                         temperature=c["T"], tf_bin_width=g["box"][0] / g["tf_bins"], rebuild_interval=g["K"], ctx=ctx)
        d.forward(table, 1.0, 1.0)  # warm-up (allocations, first rebuilds)
        d.backward()
        l0 = ctx.launches
        with ClockSampler(local_rank) as clk:
            t0 = time.perf_counter()
            loss = d.forward(table, 1.0, 1.0)
            t1 = time.perf_counter()
            gt, ge, gs = d.backward()
            t2 = time.perf_counter()
        res[form] = dict(loss=loss, fwd=t1 - t0, bwd=t2 - t1, launches=ctx.launches - l0, clocks=clk.summary(),
                         grad_eps=ge, grad_sigma=gs, grad_table_norm=float(np.linalg.norm(gt)))
        d.close()
    # the table fitted by gradient descent next to the reference's iterative
    # update, both scored with the trajectory loss (the last form)
    fit = None
    if args.fit_iterations > 0:
        from mrmd_gb300.tf_fit import ThermoForceFit

        tf = ThermoForceFit(rep, pos, vel, g["hy"], steps=g["steps"], window=g["window"],
                            checkpoint_interval=g["ckpt"], loss_bins=g["loss_bins"], loss_sigma=g["loss_sigma"],
                            tf_bin_width=g["box"][0] / g["tf_bins"], tf_target_density=c["rho"],
                            tf_modulation=c["mod"], tf_sigma=c["tfs"], tf_range=c["tfr"], capping_distance=c["cap"],
                            precision=prec, dt=c["dt"], gamma=c["gamma"], temperature=c["T"],
                            rebuild_interval=g["K"], ctx=ctx)
        t0 = time.perf_counter()
        tg, lg = tf.gradient_descent(table, args.fit_iterations)
        t1 = time.perf_counter()
        tu, lu = tf.iterative_update(table, args.fit_iterations)
        t2 = time.perf_counter()
        tf.close()
        # both tables scored on a held-out trajectory: same start, other noise
        held = M.DiffSystem(M.Replica(n, [0, 0, 0], list(g["box"]), list(g["center"]), g["at"], 4321), pos, vel,
                            hybrid_diameter=g["hy"], steps=g["steps"], window=g["window"],
                            checkpoint_interval=g["ckpt"], loss_bins=g["loss_bins"], loss_sigma=g["loss_sigma"],
                            capping_distance=c["cap"], precision=prec, dt=c["dt"], gamma=c["gamma"],
                            temperature=c["T"], tf_bin_width=g["box"][0] / g["tf_bins"], rebuild_interval=g["K"],
                            ctx=ctx)
        heldout = {k: held.forward(t, 1.0, 1.0) for k, t in
                   (("initial", table), ("gradient_descent", tg), ("iterative_update", tu))}
        held.close()
        fit = {"form": form, "iterations": args.fit_iterations, "gradient_descent_loss": lg,
               "iterative_update_loss": lu, "gradient_descent_s": t1 - t0, "iterative_update_s": t2 - t1,
               "held_out_loss": heldout,
               "note": "loss[k] before iteration k; the iterative update is ThermodynamicForce::update "
                       f"(smoothing sigma {c['tfs']}, range {c['tfr']}) after each {g['steps']}-step trajectory"}
    cpu = None
    if not args.no_cpu:
        ncores, model = cpu_info()
        geo = dict(box=g["box"], center=g["center"], at=g["at"], hy=g["hy"], K=g["K"])
        cv, done, ctime = run_adress_cpu(pos, vel, 10 ** 6, 1, args.cpu_budget, ncores, geo)
        cpu = {"value": cv, "unit": METRIC, "cores": ncores, "kind": "port",
               "sample": f"forward only: {done} steps of the {n}-molecule system by the oracle loop, "
                         f"{ncores} OpenMP threads ({model}); the reference has no adjoint"}
    head = "mixed" if "mixed" in res else next(iter(res))
    r = res[head]
    steps = g["steps"]
    value = n * steps / (r["fwd"] + r["bwd"])
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": steps, "warmup": 1,
        "ms_per_step": 1e3 * (r["fwd"] + r["bwd"]) / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if head == "fp64" else "f64 state, f32 double-float pair arithmetic",
        "data": "synthetic (seeded uniform positions, Maxwell-Boltzmann velocities)",
        "config": {"workload": DIFF_WORKLOAD, "molecules": n, "form": head,
                   "note": "value = molecules x steps / (forward + adjoint wall time) of one gradient",
                   "forms": {f: {"forward_s": res[f]["fwd"], "backward_s": res[f]["bwd"], "loss": res[f]["loss"],
                                 "atom_steps_per_s_forward": n * steps / res[f]["fwd"],
                                 "atom_steps_per_s_gradient": n * steps / (res[f]["fwd"] + res[f]["bwd"]),
                                 "dL_depsilon": res[f]["grad_eps"], "dL_dsigma": res[f]["grad_sigma"],
                                 "norm_dL_dtable": res[f]["grad_table_norm"], "kernel_launches": res[f]["launches"]}
                             for f in res},
                   "tf_fit": fit},
        "gpu_launches": r["launches"], "clocks": r["clocks"], "cpu_baseline": cpu}
    print(json.dumps(out), flush=True)


PRECISION_WORKLOAD = ("LJ fluid 4,000,000 atoms (fcc 100^3, rho 0.8442, T 0.728, rc 2.5 shifted, skin 0.3, "
                      "rebuild/10, dt 0.005), 10,000 NVE steps per form")


def precision_main(args, rank, world, local_rank):
    """The precision study: both forms run the same 4 M-atom fluid for
    `--steps` NVE steps (default 10,000) recording LJ energy and kinetic energy
    of every step on the device; energy drift per atom per 1000 tau from a
    linear fit, force error of the mixed form against FP64 at the end state."""
    import torch

    torch.cuda.set_device(local_rank)
    import mrmd_gb300 as M

    if rank != 0:
        return
    ctx = M.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    pos, L = fcc(args.cells)
    n = len(pos)
    vel = mb_velocities(n, 0.728, 1000)
    out = {}
    systems = {}
    for form in ("fp64", "mixed"):
        prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
        s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=prec, observe=True, ctx=ctx)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        rec = s.run_observed(args.steps)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        et = (rec[:, 0] + rec[:, 2]) / n
        t = np.arange(args.steps) * 0.005
        half = args.steps // 2
        out[form] = {"atom_steps_per_s": n * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "nve_drift_per_atom_per_1000tau": float(np.polyfit(t, et, 1)[0]) * 1000.0,
                     "drift_second_half": float(np.polyfit(t[half:], et[half:], 1)[0]) * 1000.0,
                     "energy_per_atom_start_end": [float(et[0]), float(et[-1])],
                     "max_abs_momentum": float(np.abs(rec[:, 3:]).max())}
        systems[form] = s
    p, v, _ = systems["fp64"].state()
    for f in systems.values():
        f.set_state(p, v)
        f.eval_forces()
    _, _, fm = systems["mixed"].state()
    _, _, fr = systems["fp64"].state()
    d = np.linalg.norm(fm - fr, axis=1)
    rms = float(np.sqrt((np.linalg.norm(fr, axis=1) ** 2).mean()))
    line = {"metric": METRIC, "value": out["mixed"]["atom_steps_per_s"], "unit": METRIC, "n_gpus": 1,
            "steps": args.steps, "warmup": 0, "ms_per_step": out["mixed"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": MIXED_DTYPE,
            "data": "synthetic (seeded fcc lattice + Maxwell-Boltzmann velocities)",
            "config": {"workload": PRECISION_WORKLOAD, "atoms": n, "forms": out,
                       "mixed_over_fp64": out["mixed"]["atom_steps_per_s"] / out["fp64"]["atom_steps_per_s"],
                       "force_error_mixed_vs_fp64_end_state": {"max_abs_over_rms": float(d.max() / rms),
                                                               "rms_over_rms": float(np.sqrt((d ** 2).mean()) / rms)}}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--workload", choices=["lj", "adress", "batch", "diff", "precision"], default="lj")
    ap.add_argument("--no-autotune", action="store_true", help="batch workload: keep the default tuning")
    ap.add_argument("--list-layout", type=int, default=0, choices=[0, 1, 2],
                    help="batch workload: list layout before autotuning (0 rows, 1 near/far rows, 2 8x4 clusters)")
    ap.add_argument("--replicas", type=int, default=None, help="batch workload: replica count (default 512)")
    ap.add_argument("--molecules", type=int, default=None,
                    help="adress workload: molecules (default 34,560; the box is scaled at density 0.5)")
    ap.add_argument("--cells", type=int, default=100, help="fcc cells per edge (100 -> 4,000,000 atoms)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-adress", action="store_true", help="lj workload: skip the AdResS sub-results")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU work for the baseline")
    ap.add_argument("--forms", default="fp64,mixed")
    ap.add_argument("--fit-iterations", type=int, default=5,
                    help="diff workload: iterations of each table fit (0 = no fit)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))

    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload == "adress":
        adress_main(args, rank, world, local_rank)
        return
    if args.workload == "batch":
        batch_main(args, rank, world, local_rank)
        return
    if args.workload == "diff":
        diff_main(args, rank, world, local_rank)
        return
    if args.workload == "precision":
        precision_main(args, rank, world, local_rank)
        return

    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    import mrmd_gb300 as M

    ctx = M.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    pos, L = fcc(args.cells)
    n = len(pos)
    vel = mb_velocities(n, 0.728, 1000 + rank)
    forms = [f.strip() for f in args.forms.split(",") if f.strip()]
    res = {}
    systems = {}

    def barrier():
        if dist is not None:
            dist.barrier()

    for form in forms:
        prec = M.PREC_MIXED if form == "mixed" else M.PREC_FP64
        sysm = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=prec, ctx=ctx)
        sysm.run(args.warmup, energies=False)
        barrier()
        with ClockSampler(local_rank) as clk:
            ms, wall, e, launches = time_run(torch, M, sysm, args.steps, stream, clk)
        ms = max_over_ranks(ms, dist, "cuda")
        res[form] = dict(ms=ms, wall=wall, launches=launches,
                         value=replica_throughput(n, args.steps, world, ms * 1e-3),
                         clocks=clk.summary(), stats=sysm.stats())
        systems[form] = sysm

    head = "mixed" if "mixed" in res else forms[0]
    sysm = systems[head]
    # the pair kernel alone (dominant kernel) for the roofline, on the state the
    # timed run left (atoms in the order of its last cell sort)
    kern_ms = time_pair_kernel(torch, sysm, stream)
    st = sysm.stats()
    tiles = sysm.tile_stats() if head == "mixed" else None

    # force error of the mixed form against FP64 on identical positions
    ferr = None
    if "mixed" in systems and "fp64" in systems:
        p, v, _ = systems["fp64"].state()
        systems["mixed"].set_state(p, v)
        systems["fp64"].set_state(p, v)
        systems["mixed"].eval_forces()
        systems["fp64"].eval_forces()
        _, _, fm = systems["mixed"].state()
        _, _, fr = systems["fp64"].state()
        d = np.linalg.norm(fm - fr, axis=1)
        mag = np.linalg.norm(fr, axis=1)
        rms = float(np.sqrt((mag ** 2).mean()))
        ferr = {"max_abs_over_rms": float(d.max() / rms), "rms_over_rms": float(np.sqrt((d ** 2).mean()) / rms),
                "max_per_atom_relative": float((d / np.maximum(mag, 1e-300)).max()),
                "max_relative_floor_0.1rms": float((d / np.maximum(mag, 0.1 * rms)).max())}

    # NVE energy drift of each form on separate equilibrated systems
    drift = nve_drift(M, ctx, list(res)) if rank == 0 else {}
    for f in res:
        res[f]["drift"] = drift.get(f, {}).get("drift")

    # the AdResS workload beside it (34,560 molecules and 4 M molecules)
    adress = None
    if rank == 0 and world == 1 and not args.no_adress:
        adress = {"workload": ADRESS_WORKLOAD,
                  "34560": adress_leg(M, ctx, torch, stream, None, list(res)),
                  "4000000": adress_leg(M, ctx, torch, stream, 4_000_000, list(res))}

    nbar = st["pairs"] / n
    # Algorithmic bytes of the pair force per atom: the half-list FP64 layout,
    # positions (24 B) read and forces (24 B) written once, one int32 count and
    # one int32 per half-list entry.  The mixed kernel moves more by design
    # (kernel_bytes_per_atom): 32-byte split records and the full list (every
    # pair from both ends, so that no force is scattered with atomics).
    nhalf = nbar / 2 if head == "mixed" else nbar
    bytes_per_atom = 24 + 24 + 4 * (1 + nhalf)
    if head == "mixed":
        # own 24-byte record, F (double4) written, near/far counts, 16-bit
        # slots of the full list, and per tile member: its index and record
        kernel_bytes = 24 + 32 + 8 + 2 * nbar + 28 * tiles["members"] / n
        kname = "lj_tile"
    else:
        kernel_bytes = bytes_per_atom
        kname = "lj_fp64"
    peak, peak_kind = load_peaks()
    achieved = bytes_per_atom * n / (kern_ms * 1e-3) / 1e9
    tpa = load_traffic(kname)
    ipa = load_traffic(kname, "thread_instructions_per_atom")

    # end to end through the public API with pinned host buffers
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hp, hv = pin(pos), pin(vel)
    outs = [pin(np.zeros((n, 3))) for _ in range(3)]
    prec = M.PREC_MIXED if head == "mixed" else M.PREC_FP64
    e2e_sys = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=prec, ctx=ctx)
    e2e_sys.run(args.warmup)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    e2e_sys.set_state(hp, hv)
    e2e_sys.run(args.steps)
    e2e_sys.state(out=outs)
    e2e_wall = time.perf_counter() - t0
    e2e_wall = max_over_ranks(e2e_wall, dist, "cuda")
    e2e_value = replica_throughput(n, args.steps, world, e2e_wall)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ncores, model = cpu_info()
        cv, done, ctime = run_cpu(pos, vel, L, 10 ** 6, 3, args.cpu_budget, ncores)
        cpu = {"value": cv, "unit": METRIC, "cores": ncores, "kind": "port",
               "sample": f"{done} steps of the {n}-atom system after 3 warm-up steps, {ncores} OpenMP threads "
                         f"({model}); CPU restatement of the reference loop"}

    if rank != 0:
        return
    r = res[head]
    line = {
        "metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": (MIXED_DTYPE if head == "mixed" else "f64"),
        "data": "synthetic (seeded fcc lattice + Maxwell-Boltzmann velocities)",
        "config": {"workload": WORKLOAD if args.cells == 100 else WORKLOAD.replace(
                       "4,000,000 atoms (fcc 100^3", f"{n:,} atoms (fcc {args.cells}^3"),
                   "atoms": n, "form": head, "l2": "inputs larger than L2 (no flush needed)",
                   "list_pairs": st["pairs"], "ghosts": st["ghosts"],
                   "forms": {f: {"atom_steps_per_s": res[f]["value"], "ms_per_step": res[f]["ms"] / args.steps,
                                 "nve_drift_per_atom_per_1000tau": res[f]["drift"],
                                 "nve_drift_sd_over_seeds": drift.get(f, {}).get("drift_sd"),
                                 "nve_drift_per_seed": drift.get(f, {}).get("drift_per_seed"),
                                 "nve_energy_fluctuation_per_atom": drift.get(f, {}).get("fluct"),
                                 "nve_momentum_max_per_atom": drift.get(f, {}).get("momentum_max"),
                                 "kernel_launches": res[f]["launches"]} for f in res},
                   "tiles": tiles, "adress": adress,
                   "mixed_over_fp64": (res["mixed"]["value"] / res["fp64"]["value"]) if {"mixed", "fp64"} <= res.keys() else None,
                   "force_error_mixed_vs_fp64": ferr,
                   "nve_drift_measurement": DRIFT_SETUP},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(48 * n / args.steps),
                "d2h_bytes_per_step": int(16 + 72 * n / args.steps)},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "kernel_ms": kern_ms,
                     "algorithmic_bytes_per_atom": bytes_per_atom, "kernel_bytes_per_atom": kernel_bytes,
                     "kernel_bytes_gbs": kernel_bytes * n / (kern_ms * 1e-3) / 1e9,
                     "traffic": (tpa * n) if tpa is not None else None,
                     "instruction_issue": issue_roofline(torch, local_rank, ipa, n, kern_ms, r["clocks"])},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
