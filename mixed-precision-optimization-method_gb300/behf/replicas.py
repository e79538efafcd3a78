"""Replicas across processes (one GPU each): the path does not shard, independent shots do.

The grid of one shot stays on one GPU; several GPUs (or processes) run independent replicas -- the benchmark's
weak scaling -- or divide a set of shots between them, with no collective on the data path.  The only
exchanges are host-side and happen once: the maximum of the ranks' timed regions, and the sum of the ranks'
gradients of a multi-shot misfit.  These helpers work with any torch.distributed process group (NCCL on GPUs,
gloo on CPU; the tests run them as two gloo ranks).

    python -m behf.replicas --shots 16 [--n 256] [--steps 2000]      (under torchrun for several GPUs)

runs the multi-shot gradient of the inversion workload: every rank takes its share of the shots, computes
their L2-misfit gradients against the true model's data, and rank 0 prints the summed misfit and the norms of
the summed moduli gradients.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np


def shard(items: int, rank: int, world: int) -> list[int]:
    """The items (shots) of one rank: round-robin, so every item goes to exactly one rank and the ranks'
    counts differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(range(rank, items, world))


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over the ranks (the slowest rank's timed region); the value itself alone."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(arr: np.ndarray, device=None) -> np.ndarray:
    """Element-wise sum of a host array over the ranks (the multi-shot gradient); a copy when alone."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return np.array(arr, copy=True)
    import torch

    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)).to(device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


def multishot_gradient(shots: list[int], n: int, nt: int, precision: str = "f16") -> tuple[float, np.ndarray]:
    """Summed L2 misfit and moduli gradient of the given shots of the inversion workload (this rank's share)."""
    from . import problems, solver_for

    J, gm = 0.0, None
    for shot in shots:
        s = solver_for(problems.inversion256(n=n, nt=nt, shot=shot, true_model=True), precision=precision)
        s.run(nt)
        dobs = s.seismograms()
        s.close()
        s = solver_for(problems.inversion256(n=n, nt=nt, shot=shot, true_model=False), precision=precision,
                       gradient=True)
        j, _, g = s.misfit_gradient(nt, dobs)
        s.close()
        J += j
        gm = g if gm is None else gm + g
    if gm is None:
        gm = np.zeros((9, n, n, n))
    return J, gm


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--shots", type=int, default=16)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--precision", default="f16")
    args = ap.parse_args(argv)
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    mine = shard(args.shots, rank, world)
    t0 = time.perf_counter()
    J, gm = multishot_gradient(mine, args.n, args.steps, args.precision)
    sec = max_over_ranks(time.perf_counter() - t0, device="cuda" if world > 1 else None)
    dev = "cuda" if world > 1 else None
    J = float(sum_over_ranks(np.array([J]), device=dev)[0])
    gm = sum_over_ranks(gm, device=dev)
    if rank == 0:
        from . import MODULI

        print(json.dumps({"shots": args.shots, "ranks": world, "n": args.n, "steps": args.steps,
                          "precision": args.precision, "seconds": sec, "seconds_per_shot": sec * world / args.shots,
                          "misfit": J, "grad_norms": {m: float(np.linalg.norm(gm[i])) for i, m in enumerate(MODULI)}}))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
