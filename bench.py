#!/usr/bin/env python
"""Benchmark of the BEHF time stepper: Gpt-updates/s of the 1024^3 FP16 random-medium workload.

One step = one time step (source, velocity update, stress update, receiver gather) over the whole
1024^3 grid: the random heterogeneous sandstone (5 % Gaussian-correlated perturbations, log-normal
permeability), vertical-force 20 Hz source, 512 x 512 surface receivers recording vz and p, radius-4
(8th-order) stencil, 20-cell CPML.  The medium is generated on the device (synthetic data).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl behf|reference]

Timing: W untimed steps, then exactly K steps between CUDA events on the library's stream, with a
barrier + synchronize on both sides, max over ranks.  The working set (~96 GB) is far above the
129 MB L2, so no flush is needed between steps.  Multi-GPU runs independent replicas (one grid per
GPU, no collective on the data path): value = all cells updated / max time ("weak" scaling).

--impl reference times the CPU restatement of the reference's scheme (FP64, OpenMP, all host cores)
on a bounded sample of the same workload (a 160^3 grid of the same medium and scheme).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG_DIR = ROOT / "mixed-precision-optimization-method_gb300"
for _p in (str(ROOT), str(PKG_DIR)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Gpt-updates/s (1024^3 FP16 BEHF, seis relL2<=2e-2)"
UNIT = "Gpt/s"

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per updated cell of one launch of the radius-4 FP16
# tensor-memory kernels (variant 4 with the x slabs staged, the FP16 default; variant 3 without), from ncu captures
# of a 384^3 grid with a 7-cell CPML (the same slab fraction of the grid as 20 cells at 1024^3; one kernel and two
# launches per capture, 5 GB on the device); the bench multiplies by the cells of its own grid.
NCU_BYTES_PER_CELL = {("f16", "tmem_xs", "velocity"): 81.73, ("f16", "tmem_xs", "stress"): 65.30,
                      ("f16", "tmem", "velocity"): 84.57, ("f16", "tmem", "stress"): 68.47}
NCU_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per cell of one 384^3 launch with a 7-cell CPML "
              "(profiles/traffic_k_vel_zq_k_str_zq_random384_f16.md), x cells")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="behf", choices=["behf", "reference"])
    ap.add_argument("--n", type=int, default=1024, help="grid cells per axis")
    ap.add_argument("--nx", type=int, default=0, help="diagnostics: x extent of a narrower grid (0: n); nx = 128 makes "
                    "every x tile an x-edge tile")
    ap.add_argument("--cpml", type=int, default=20, help="CPML cells per face (20 at 1024^3; 7 at 384^3 gives the "
                    "same slab fraction of the grid)")
    ap.add_argument("--precision", default="f16", choices=["f16", "bf16", "f32", "f64"])
    ap.add_argument("--kernel", default="auto", choices=["auto", "plain", "tiled"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true", help="skip the FP32 comparison run")
    ap.add_argument("--cpu-n", type=int, default=160, help="grid of the CPU sample")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the gradient (adjoint) measurement")
    ap.add_argument("--adjoint-n", type=int, default=256, help="grid of the gradient measurement")
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--no-shots", action="store_true", help="skip the batched-shots measurement")
    ap.add_argument("--shots-per-size", type=int, default=16)
    ap.add_argument("--shots-steps", type=int, default=1500)
    ap.add_argument("--adjoint-only", action="store_true",
                    help="only the gradient measurement (one JSON object with the adjoint leg)")
    return ap.parse_args()


# ----------------------------------------------------------------------------- environment
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int):
        self.dev = dev
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU side
def cpu_rate(n: int, steps: int, warmup: int):
    """Oracle (FP64, OpenMP, all host cores) on an n^3 grid of the same scheme and medium."""
    from behf import problems
    from oracle import pyoracle
    prob = problems.random1024(n=n, nt=warmup + steps, cpml=min(20, n // 8), nrec_side=min(64, n // 4))
    pyoracle.run(prob, "f64", nthreads=0, time_from_step=warmup)
    sec = pyoracle.last_step_seconds()
    return n ** 3 * steps / sec / 1e9, pyoracle.threads(), sec


def reference_arm(args, world, rank):
    if rank != 0:
        return
    steps = max(args.steps, 1)
    value, cores, sec = cpu_rate(args.cpu_n, steps, args.warmup)
    sample = (f"{args.cpu_n}^3 grid of the same medium/scheme (radius 4, 20-cell CPML scaled), FP64, "
              f"{steps} timed steps after {args.warmup} warm-up, {sec:.2f} s")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": steps, "warmup": args.warmup, "ms_per_step": sec / steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config_dict(args),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def config_dict(args):
    nx = args.nx or args.n
    shape = f"{args.n}^3" if nx == args.n else f"{nx}x{args.n}x{args.n}"
    return {"workload": f"random{args.n}: {shape} cells, h=5 m, dt=0.4 ms, radius 4, {args.cpml}-cell CPML, "
                        "5% Gaussian-correlated sandstone, force source 20 Hz, 512x512 receivers (vz,p)",
            "grid": [nx, args.n, args.n], "storage": args.precision, "kernel": args.kernel,
            "parallelism": f"replicas x{args.gpus}", "l2": "no flush: working set ~96 GB >> 129 MB L2"}


# ----------------------------------------------------------------------------- GPU side
def make_solver(prob, precision, kernel, capacity):
    import behf
    s = behf.Solver(prob.nx, prob.ny, prob.nz, prob.h, prob.dt, radius=prob.radius, precision=precision,
                    cpml_width=prob.cpml_width, cpml_v0=prob.cpml_v0, cpml_r=prob.cpml_r,
                    src_amp_hint=float(np.abs(prob.wavelet).max()), src_f0_hint=prob.f0)
    s.set_kernel(kernel)
    s.generate_medium(prob.extra["spec"])
    s.set_source(prob.src_kind, prob.src, prob.wavelet)
    s.set_receivers(prob.rec_ijk, prob.rec_comp, capacity)
    return s


def timed_steps(s, steps, world):
    import torch
    st = torch.cuda.ExternalStream(s.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = s.info()["launches"]
    e0.record(st)
    s.run_async(steps)
    e1.record(st)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    launches = s.info()["launches"] - l0
    if world > 1:
        from behf import replicas

        ms = replicas.max_over_ranks(ms, device="cuda")
    return ms, launches


def adjoint_leg(args):
    """Seconds per shot of the checkpointed adjoint-state gradient (L2 misfit of vz and p) against the same
    forward run alone, on the inversion workload (256^3, 2000 steps, FP16 storage, FP32 adjoint)."""
    import torch

    import behf
    from behf import problems
    n, nt = args.adjoint_n, args.adjoint_steps
    s = behf.solver_for(problems.inversion256(n=n, nt=nt, true_model=True), precision=args.precision)
    s.run(nt)
    dobs = s.seismograms()
    s.close()
    prob = problems.inversion256(n=n, nt=nt, true_model=False)
    s = behf.solver_for(prob, precision=args.precision, gradient=True)
    s.run(min(nt, 40))  # warm-up: graph capture, first launches
    s.reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(nt)
    t1 = time.perf_counter()
    s.reset()
    l0 = s.info()["launches"]
    t2 = time.perf_counter()
    J, gw, gm = s.misfit_gradient(nt, dobs)
    t3 = time.perf_counter()
    launches = s.info()["launches"] - l0
    s.close()
    fwd, grad = t1 - t0, t3 - t2
    return {"workload": f"inversion{n}: {n}^3 two-layer medium, anomaly-free start model, explosive (pressure) "
                        f"source 25 Hz, "
                        f"{len(prob.rec_comp)} traces (vz, p), L2 misfit",
            "steps": nt, "storage": args.precision, "adjoint_arithmetic": "f64" if args.precision == "f64" else "f32",
            "checkpoint_every": int(round(nt ** 0.5)), "forward_s": fwd, "gradient_s_per_shot": grad,
            "gradient_over_forward": grad / fwd, "misfit": J, "gpu_launches": int(launches),
            "grad_norms": {k: float(np.linalg.norm(gm[i])) for i, k in
                           enumerate(("rho", "rhof", "mu", "M", "C", "HH", "H2U", "C1", "C2"))}}


def shots_leg(args):
    """Many independent shots on one GPU (48 shots: 16 each of 128^3, 192^3, 256^3, 1500 steps, FP16, radius 4,
    20-cell CPML, layered + random medium from each shot's seed, 30 Hz explosive (pressure) source at a seeded
    position, 128 receivers): batched on overlapping streams (behf_run_batch, graph-captured time loop) with the kernel variant
    and z range the autotuner picked for each size, against the same shots run one after another with the default
    kernels.  Medium generation is outside the timed regions."""
    import torch

    import behf
    from behf import shots
    sizes = [128, 192, 256]
    per, nt, batch = args.shots_per_size, args.shots_steps, 4
    cells_steps = sum(n ** 3 for n in sizes) * per * nt
    t_seq, t_bat, tuned, launches = 0.0, 0.0, {}, 0
    for n in sizes:
        s = behf.solver_for(shots.shot_problem(n, 1000 * n, nt), precision=args.precision)
        z, ms = s.autotune(3)
        tuned[n] = {"variant": s.info()["tiled_variant"], "tile_rows": s.info()["tile_rows"], "zchunk": z,
                    "ms_per_step": ms}
        s.close()
        for i in range(per):
            s = behf.solver_for(shots.shot_problem(n, 1000 * n + i, nt), precision=args.precision)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run(nt)
            t_seq += time.perf_counter() - t0
            s.close()
        for g0 in range(0, per, batch):
            group = [behf.solver_for(shots.shot_problem(n, 1000 * n + i, nt), precision=args.precision)
                     for i in range(g0, min(per, g0 + batch))]
            for s in group:
                s.set_option(behf.OPT_TILE_ROWS, tuned[n]["tile_rows"])
                s.set_option(behf.OPT_TILED_VARIANT, behf.TILED_VARIANT[tuned[n]["variant"]])
                s.set_option(behf.OPT_ZCHUNK, tuned[n]["zchunk"])
            l0 = sum(s.info()["launches"] for s in group)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            behf.run_batch(group, nt)
            t_bat += time.perf_counter() - t0
            launches += sum(s.info()["launches"] for s in group) - l0
            for s in group:
                s.close()
    return {"workload": f"{per} shots each of {sizes} cells per axis, {nt} steps, {args.precision}, radius 4, "
                        "20-cell CPML, layered + random medium per shot, explosive (pressure) source 30 Hz, "
                        "128 receivers",
            "sequential_s": t_seq, "batched_s": t_bat, "sequential_gpts": cells_steps / t_seq / 1e9,
            "batched_gpts": cells_steps / t_bat / 1e9, "batched_over_sequential": t_seq / t_bat,
            "batch": batch, "autotuned": tuned, "gpu_launches_batched": int(launches)}


def behf_arm(args, world, rank, local):
    import torch

    import behf
    from behf import problems

    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    n = args.n
    ktime = 3
    e2e_steps = 0 if args.no_e2e else max(args.steps // 2, 3)
    total = args.warmup + args.steps + ktime + e2e_steps
    prob = problems.random1024(n=n, nt=total, medium=False, cpml=args.cpml)
    nx = args.nx or n
    if nx != n:  # a narrower grid: the x extent cut, the source and receivers moved inside it
        ijk = prob.rec_ijk.copy()
        ijk[:, 0] = np.clip(ijk[:, 0], args.cpml + 2, nx - args.cpml - 3)
        prob = dataclasses.replace(prob, nx=nx, src=(nx // 2,) + tuple(prob.src[1:]), rec_ijk=ijk)
    cells = prob.cells
    s = make_solver(prob, args.precision, args.kernel, total)
    s.run(args.warmup)
    sampler = ClockSampler(local)
    sampler.start()
    ms, launches = timed_steps(s, args.steps, world)
    clocks = sampler.stop()
    value = world * cells * args.steps / (ms * 1e-3) / 1e9
    ok, _ = s.health()

    # per-kernel durations (CUDA events around each launch, on the library's stream)
    kt = s.time_kernels(ktime)
    ab = behf.algorithmic_bytes(args.precision, (nx, n, n), prob.cpml_width)
    dom = "velocity" if kt["velocity"] >= kt["stress"] else "stress"
    peak, peak_kind = peak_hbm()
    achieved = ab[dom] * cells / (kt[dom] * 1e-3) / 1e9
    info = s.info()
    bpc = (NCU_BYTES_PER_CELL.get((args.precision, info["tiled_variant"], dom))
           if info["kernel"] == "tiled" and prob.radius == 4 else None)
    traffic = bpc * cells if bpc is not None else None
    traffic_src = NCU_SOURCE if bpc is not None else None

    # end to end through the C ABI with host buffers: per step, the wavelet sample goes host->device
    # (pinned) and the step's seismogram column (every receiver) comes back device->host (pinned)
    e2e = None
    if e2e_steps:
        it0 = args.warmup + args.steps + ktime
        w_host = torch.from_numpy(prob.wavelet.copy()).pin_memory().numpy()
        col = torch.zeros((s.nrec, 1), dtype=torch.float64).pin_memory().numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for it in range(it0, it0 + e2e_steps):
            s.update_wavelet(it, w_host[it:it + 1])
            s.run(1)
            s.seismograms_range(it, 1, col)
        t1 = time.perf_counter()
        e2e_val = world * cells * e2e_steps / (t1 - t0) / 1e9
        e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 4, "d2h_bytes_per_step": int(s.nrec * 8),
               "steps": e2e_steps}
    s.close()
    del s

    fp32 = None
    if not args.no_fp32 and args.precision in ("f16", "bf16") and rank == 0:
        # the same workload stored in FP32 (same kernels, FP32 instantiation) and the plain FP32 kernel
        fp32 = {}
        for kern in ("auto", "plain"):
            s32 = make_solver(prob, "f32", kern, total)
            s32.run(2)
            k = max(args.steps // 2, 4)
            ms32, _ = timed_steps(s32, k, 1)
            fp32[kern] = cells * k / (ms32 * 1e-3) / 1e9
            fp32[kern + "_kernel"] = s32.info()["kernel"]
            s32.close()
            del s32

    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = adjoint_leg(args)

    shots_out = None
    if rank == 0 and not args.no_shots:
        shots_out = shots_leg(args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, sec = cpu_rate(args.cpu_n, 6, 1)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_n}^3 grid of the same medium and scheme, FP64 OpenMP, 6 steps ({sec:.1f} s)"}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": args.precision, "data": "synthetic (device-generated random medium)",
               "config": config_dict(args), "e2e": e2e, "gpu_launches": int(launches),
               "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                            "peak_source": peak_kind,
                            "bytes_per_cell": ab[dom], "kernel_ms": kt[dom]},
               "step_roofline": {"bytes_per_cell_fused": ab["step_fused"], "bytes_per_cell_unfused": ab["step_unfused"],
                                 "achieved": value / world * ab["step_fused"], "frac": value / world * ab["step_fused"] / peak,
                                 "roofline_gpts": peak / ab["step_fused"]},
               "kernel_ms": kt, "kernel_family": info["kernel"], "kernel_variant": info["tiled_variant"],
               "tile_rows": info["tile_rows"],
               "scales": info["scales"], "health_ok": ok,
               "fp32": fp32, "fp16_over_fp32": (value / world / fp32["auto"]) if fp32 else None,
               "fp16_over_plain_fp32": (value / world / fp32["plain"]) if fp32 else None,
               "clocks": clocks, "cpu_baseline": cpu, "device_bytes": info["device_bytes"], "adjoint": adjoint,
               "shots": shots_out}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
        return
    import behf
    behf.load()
    if args.adjoint_only:
        if rank == 0:
            import torch
            torch.cuda.set_device(local)
            print(json.dumps({"adjoint": adjoint_leg(args)}), flush=True)
        return
    behf_arm(args, world, rank, local)


if __name__ == "__main__":
    main()
