"""A plain run of the fused LJ stepper for profiler captures and phase timing.

    python -m mrmd_gb300.profile_run [--cells 40] [--steps 20] [--warmup 5]
                                     [--form mixed|fp64] [--gather] [--kernel-reps 10]
                                     [--sort 4]

Builds the fcc LJ fluid of the benchmark (cells^3 unit cells, rho 0.8442,
T 0.728), runs `warmup` steps, then `steps` steps, then launches the pair
kernel alone `kernel-reps` times.  It starts no helper process (no clock
sampling), so that a profiler attached to it sees this process only.  It
prints one JSON line with CUDA-event times of the phases: the run per step,
the pair kernel, and one full rebuild with its force evaluation.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def fcc(cells, rho=0.8442):
    a = (4.0 / rho) ** (1.0 / 3.0)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(cells)] * 3, indexing="ij"), -1).reshape(-1, 3)
    return ((g[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25) * a, a * cells


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=40)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--form", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--gather", action="store_true", help="mixed form: gather records instead of tiles")
    ap.add_argument("--kernel-reps", type=int, default=10)
    ap.add_argument("--sort", type=int, default=4, help="re-sort the atoms at every k-th rebuild")
    args = ap.parse_args()

    import torch

    import mrmd_gb300 as M

    ctx = M.default_context()
    stream = torch.cuda.ExternalStream(ctx.stream)
    pos, L = fcc(args.cells)
    n = len(pos)
    rng = np.random.default_rng(1000)
    vel = rng.normal(0.0, np.sqrt(0.728), (n, 3))
    vel -= vel.mean(0)
    prec = M.PREC_MIXED if args.form == "mixed" else M.PREC_FP64
    s = M.LJSystem(pos, vel, [0, 0, 0], [L] * 3, precision=prec, gather_neighbours=args.gather,
                   sort_atoms=args.sort, ctx=ctx)
    s.run(args.warmup, energies=False)

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ctx.sync()
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    run_ms = timed(lambda: s.run(args.steps, energies=False))
    kernel_ms = 0.0
    if args.kernel_reps > 0:
        kernel_ms = timed(lambda: [s.launch_pair_kernel() for _ in range(args.kernel_reps)]) / args.kernel_reps
    # one rebuild (ghosts, cell sort, list, tiles) with its force evaluation
    p, v, _ = s.state()
    s.set_state(p, v)
    rebuild_ms = timed(lambda: s.eval_forces())
    out = {"atoms": n, "form": args.form, "steps": args.steps, "ms_per_step": run_ms / args.steps,
           "pair_kernel_ms": kernel_ms, "rebuild_and_forces_ms": rebuild_ms, "stats": s.stats()}
    if args.form == "mixed":
        out["tiles"] = s.tile_stats()
    print(json.dumps(out), flush=True)
    s.close()


if __name__ == "__main__":
    main()
