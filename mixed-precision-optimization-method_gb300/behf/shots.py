"""Many independent shots on one GPU: sequential runs against batched runs (behf_run_batch).

    python -m behf.shots [--per-size 16] [--sizes 128,192,256] [--steps 1500] [--batch 4] [--precision f16]

The shot workload: per grid size, `per-size` shots, each its own medium (two layers with the interface at
mid-depth, 5 % Gaussian-correlated perturbations from the shot's seed), a 30 Hz explosive (pressure) source at a
seeded random position 6 cells below the top CPML, 128 receivers (vz, p) on a surface line, 20-cell CPML,
radius 4.  Set-up (medium generation, coefficients) is outside the timed region; the time is the run only.
Prints one JSON object: Gpt-updates/s sequential, batched, and the autotuned z-chunk of each size.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import run_batch, solver_for
from . import problems as P


def shot_problem(n: int, seed: int, nt: int = 1500, cpml: int = 20) -> P.Problem:
    h, dt, f0 = 5.0, 4e-4, 30.0
    rng = np.random.default_rng(seed)
    sx, sy = (int(v) for v in rng.integers(cpml + 6, n - cpml - 6, size=2))
    spec = dict(layers=[P.SANDSTONE, P.STIFF], interfaces=(n // 2,), seed=seed % (1 << 20), corr_cells=10.0,
                pct=0.05, log_kappa_sigma=0.5, anomaly=None)
    xs = np.linspace(cpml + 2, n - cpml - 3, 64).round().astype(int)
    ijk, comp = P.line_receivers(xs, n // 2, cpml + 2, [2, 12])
    return P.Problem(n, n, n, h, dt, 4, np.zeros((9, 1, 1, 1), np.float32), P.ricker(nt, dt, f0),
                     (sx, sy, cpml + 6), ijk, comp, src_kind="explosive", cpml_width=cpml,
                     cpml_v0=P.p_velocity(P.STIFF), f0=f0, name=f"shot{n}_{seed}", extra={"spec": spec})


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="128,192,256")
    ap.add_argument("--per-size", type=int, default=16)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--precision", default="f16")
    args = ap.parse_args(argv)
    sizes = [int(v) for v in args.sizes.split(",")]
    out = {"workload": f"{args.per_size} shots per size {sizes}, {args.steps} steps, radius 4, 20-cell CPML, "
                       f"explosive (pressure) source 30 Hz, 128 receivers", "precision": args.precision,
           "batch": args.batch}
    cells_steps = sum(n ** 3 for n in sizes) * args.per_size * args.steps
    # sequential
    t_seq, tune = 0.0, {}
    for n in sizes:
        for i in range(args.per_size):
            s = solver_for(shot_problem(n, 1000 * n + i, args.steps), precision=args.precision)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run(args.steps)
            t_seq += time.perf_counter() - t0
            s.close()
        s = solver_for(shot_problem(n, 1000 * n, args.steps), precision=args.precision)
        tune[n] = s.autotune(4)
        s.close()
    # batched: groups of `batch` shots of one size on their own streams
    t_bat = 0.0
    for n in sizes:
        for g0 in range(0, args.per_size, args.batch):
            group = [solver_for(shot_problem(n, 1000 * n + i, args.steps), precision=args.precision)
                     for i in range(g0, min(args.per_size, g0 + args.batch))]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            run_batch(group, args.steps)
            t_bat += time.perf_counter() - t0
            for s in group:
                s.close()
    out.update({"sequential_s": t_seq, "batched_s": t_bat, "sequential_gpts": cells_steps / t_seq / 1e9,
                "batched_gpts": cells_steps / t_bat / 1e9, "autotune_zchunk_ms": tune})
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
