"""Full-size accuracy of the storage precisions: seismogram relative L2 per recorded field and, except at 1024^3,
the relative L2 of each of the 13 final wavefields.

    python -m behf.accuracy --workload layered256 [--steps 2000]
        FP64 (the plain kernels, the GPU oracle run of the same scheme) vs FP32, FP16, BF16 (tiled kernels)
    python -m behf.accuracy --workload random1024 [--steps 1200]
        FP16 and BF16 vs FP32 (FP64 at 1024^3 does not fit one GPU; FP32 is within 1e-4 of FP64 on the
        parity tests, so the FP16-vs-FP32 error stands for FP16-vs-FP64)
    python -m behf.accuracy --workload borehole [--steps 3500]
        the reference's own problem (240 x 240 x 360 cells of 1 cm, fluid-filled borehole, R = 1, 10 kHz,
        bug-compatible vz, the reference's storage scales, txx on the vertical line through the source):
        FP64 vs FP32, FP16, BF16 (automatic scales; --ref-scales: the reference's 1e8, 1e8, 1, 1)

Prints one JSON object: per precision and per recorded field the relative L2 error of all traces (and in the
signal band, both traces low-passed at 4 f0), per
wavefield the relative L2 error of the field after nt/4, nt/2 and nt steps (physical units, read back as float32;
`field_rel_l2` is the final one; with the reference's field norms at those steps, since a field whose waves have
left through the CPML is a small residue whose relative error says little; skipped at 1024^3, where 13 fields are
56 GB of host memory per run), the storage scales, the wall time, and the health check (NaN/Inf/saturation) at
the end.  Runs the precisions one after another (one context on the device at a time).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import FIELDS, solver_for
from . import problems


def run_one(prob, precision: str, kernel: str = "auto", coef_rounding: int = 0, state_rounding: int = 0,
            scale_boost: int = 0, fields: bool = False, scales=None):
    half = precision in ("f16", "bf16")
    if scale_boost and half:  # the automatic scales times 2^scale_boost
        s0 = solver_for(prob, precision, kernel)
        scales = [v * 2.0 ** scale_boost for v in s0.info()["scales"]]
        s0.close()
    s = solver_for(prob, precision, kernel, scales=scales, coef_rounding=coef_rounding if half else 0,
                   state_rounding=state_rounding if half else 0)
    # wavefield snapshots after nt/4, nt/2 and nt steps (the time loop is timed without the read-backs)
    marks = sorted({max(1, prob.nt // 4), max(1, prob.nt // 2), prob.nt}) if fields else [prob.nt]
    snaps, wall, done = {}, 0.0, 0
    for m in marks:
        t0 = time.perf_counter()
        s.run(m - done)
        wall += time.perf_counter() - t0
        done = m
        if fields:
            snaps[m] = {name: s.get_field(name) for name in FIELDS}
    seis = s.seismograms()
    ok, _ = s.health()
    info = s.info()
    s.close()
    return seis, {"wall_s": wall, "health_ok": bool(ok), "kernel": info["kernel"], "scales": info["scales"],
                  "gpts": prob.cells * prob.nt / wall / 1e9}, snaps if fields else None


def lowpass(x: np.ndarray, dt: float, fc: float) -> np.ndarray:
    """Zero-phase low-pass of each trace (rows): the FFT bins above fc set to zero."""
    X = np.fft.rfft(x, axis=1)
    X[:, np.fft.rfftfreq(x.shape[1], dt) > fc] = 0
    return np.fft.irfft(X, n=x.shape[1], axis=1)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / den) if den > 0 else float("nan")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="layered256", choices=["layered256", "random1024", "small64", "borehole"])
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--n", type=int, default=0, help="grid override (test-sized runs)")
    ap.add_argument("--coef-rounding", type=int, default=0, help="1: unbiased coefficient rounding (16-bit kinds)")
    ap.add_argument("--state-rounding", type=int, default=0, help="1: stochastic rounding of the stored fields")
    ap.add_argument("--scale-boost", type=int, default=0, help="16-bit kinds: automatic scales times 2^B")
    ap.add_argument("--no-fields", action="store_true", help="skip the final-wavefield errors")
    ap.add_argument("--ref-scales", action="store_true",
                    help="borehole: the reference's storage scales (1e8, 1e8, 1, 1) instead of the automatic ones")
    args = ap.parse_args(argv)
    if args.workload == "layered256":
        prob = problems.layered256(n=args.n or 256, nt=args.steps or 2000)
        ref_prec, others = "f64", ["f32", "f16", "bf16"]
    elif args.workload == "borehole":
        prob = problems.borehole(scale=args.n / 180 if args.n else 1.0, nt=args.steps or 3500)
        ref_prec, others = "f64", ["f32", "f16", "bf16"]
    elif args.workload == "small64":
        prob = problems.small64(n=args.n or 64, nt=args.steps or 500)
        ref_prec, others = "f64", ["f32", "f16", "bf16"]
    else:
        prob = problems.random1024(n=args.n or 1024, nt=args.steps or 1200, medium=False, nrec_side=128)
        ref_prec, others = "f32", ["f16", "bf16"]
    out = {"workload": prob.name, "cells": prob.cells, "steps": prob.nt, "reference": ref_prec, "runs": {},
           "coef_rounding": args.coef_rounding, "state_rounding": args.state_rounding,
           "scale_boost": args.scale_boost}
    scales = None
    if args.ref_scales:
        if args.workload != "borehole":
            ap.error("--ref-scales applies to the borehole workload")
        scales = prob.scales
        out["scales"] = "reference"
    fields = not args.no_fields and args.workload != "random1024"
    ref, meta, ref_fields = run_one(prob, ref_prec, fields=fields, scales=scales)
    if fields:  # L2 norm of each reference field at each snapshot step (how much of the wave is still inside)
        meta["field_norm"] = {m: {name: float(np.linalg.norm(f[name].astype(np.float64).ravel())) for name in FIELDS}
                              for m, f in ref_fields.items()}
    out["runs"][ref_prec] = meta
    comps = np.unique(prob.rec_comp)
    out["peak"] = {FIELDS[c]: float(np.abs(ref[prob.rec_comp == c]).max()) for c in comps}
    for prec in others:
        seis, meta, final = run_one(prob, prec, coef_rounding=args.coef_rounding,
                                    state_rounding=args.state_rounding, scale_boost=args.scale_boost, fields=fields,
                                    scales=scales)
        meta["rel_l2"] = {FIELDS[c]: rel_l2(seis[prob.rec_comp == c], ref[prob.rec_comp == c]) for c in comps}
        # the same in the signal band (both traces low-passed at 4 f0, which keeps the reference's energy)
        fc = 4 * prob.f0
        meta["rel_l2_band"] = {FIELDS[c]: rel_l2(lowpass(seis[prob.rec_comp == c], prob.dt, fc),
                                                 lowpass(ref[prob.rec_comp == c], prob.dt, fc)) for c in comps}
        if fields:
            meta["field_rel_l2_at"] = {m: {name: rel_l2(final[m][name], ref_fields[m][name]) for name in FIELDS}
                                       for m in ref_fields}
            meta["field_rel_l2"] = meta["field_rel_l2_at"][prob.nt]
        out["runs"][prec] = meta
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
