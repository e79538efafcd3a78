"""Generate the golden fixtures of the reference's own kernels (run where the reference tree exists).

The reference publishes no test vectors, so these fixtures come from running the reference's
``Source``/``FD_Vbottom``/``FD_Tbottom`` kernel bodies and its ``create_model_all`` medium builder,
compiled for the CPU by ``oracle/build.py`` (``oracle/_ref``), on small single-domain problems:

* ``ref_borehole.npz`` -- the reference's own borehole medium (outputfunc.cpp:153-222),
  h = 1 cm, dt = 1 us, 10 kHz Ricker, explosive source, 5-cell CPML.
* ``ref_rock.npz`` -- a seeded heterogeneous porous rock (Biot-Gassmann moduli of a sandstone
  with 10 % random perturbations), same scheme.

Each file holds the FP16 inputs (coefficients, CPML profiles, wavelet), the receiver list and the
reference outputs after ``nt`` steps: the 16 state arrays, the 48 CPML arrays and the seismograms.
Usage: ``python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import pyoracle as po  # noqa: E402

OUT = Path(__file__).resolve().parent


def ricker_ref(nt: int, dt: float, f0: float) -> np.ndarray:
    """Ricker samples as kernel.cu:1898 forms them (float tt, float T0, double expression)."""
    t0 = np.float32(1.2 / f0)
    w = np.zeros(nt, np.float32)
    for it in range(nt):
        tt = np.float32(it * np.float32(dt))
        a = np.pi * np.pi * f0 * f0 * float(tt - t0) * float(tt - t0)
        w[it] = np.float32(-(1 - 2 * a) * np.exp(-a))
    return w


def rock_medium(nz, ny, nx, seed):
    rng = np.random.default_rng(seed)
    mod = np.zeros((po.NMOD, nz, ny, nx), np.float32)
    base = dict(Ks=37e9, Kf=2.25e9, Kdry=9e9, mu=7e9, rhos=2650.0, rhof=1000.0, phi=0.2, kappa=1e-12, eta=1e-3,
                tau=2.4)
    pk = rng.uniform(-0.1, 0.1, size=(4, nz, ny, nx))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                p = dict(base)
                p["Kdry"] *= 1 + pk[0, k, j, i]
                p["mu"] *= 1 + pk[1, k, j, i]
                p["phi"] *= 1 + pk[2, k, j, i]
                p["kappa"] *= np.exp(pk[3, k, j, i] * 5)
                mod[:, k, j, i] = po.rock_moduli(**p)
    return mod


def make_case(name, mod, np_cells, nt, src, recs):
    _, nz, ny, nx = mod.shape
    h, dt, f0 = 0.01, 1e-6, 1e4
    coef, prof = po.ref_inputs(mod, h, dt, np_cells)
    w = ricker_ref(nt, dt, f0)
    sx, sy, sz = src
    sn = (sz * ny + sy) * nx + sx
    rec_lin = np.array([(k * ny + j) * nx + i for (i, j, k, _) in recs], np.int32)
    rec_comp = np.array([c for (*_, c) in recs], np.int32)
    state = np.zeros((16, nz, ny, nx), np.uint16)
    aux = np.zeros((48, nz, ny, nx), np.uint16)
    seis = po.ref_run((nz, ny, nx), dt, nt, sn, w, state, coef, prof, aux, rec_lin, rec_comp, use_reference=True)
    np.savez_compressed(OUT / f"{name}.npz", shape=np.array([nz, ny, nx]), h=h, dt=dt, f0=f0, np_cells=np_cells,
                        nt=nt, sn=sn, src=np.array(src), wavelet=w, coef=coef, prof=prof, medium=mod,
                        rec_lin=rec_lin, rec_comp=rec_comp, state=state, aux=aux, seis=seis)
    print(name, "max|seis|", float(np.abs(seis).max()), "bytes", (OUT / f"{name}.npz").stat().st_size)


def main():
    if po.ref_lib() is None:
        raise SystemExit("reference tree not available: fixtures can only be regenerated where it is")
    nz, ny, nx = 18, 30, 32
    mod = po.ref_medium(nz, ny, nx)
    recs = [(nx // 2 + 11, ny // 2, k, 6) for k in range(2, nz - 2)]          # txx line beside the borehole
    recs += [(nx // 2 + 12, ny // 2 + 3, nz // 2, c) for c in range(13)]      # every field at one point
    make_case("ref_borehole", mod, 5, 60, (nx // 2 + 12, ny // 2, nz // 2), recs)
    nz, ny, nx = 16, 18, 20
    mod = rock_medium(nz, ny, nx, seed=7)
    recs = [(i, 9, 8, c) for i in range(3, 17, 3) for c in (2, 5, 12)]
    make_case("ref_rock", mod, 4, 50, (9, 8, 7), recs)


if __name__ == "__main__":
    main()
