"""ctypes front end of the CPU oracle (test infrastructure, the checker of the CUDA path).

Only the tests, the smoke check and the benchmark's CPU-baseline leg import this module.
It wraps ``oracle/_build/liboracle.so`` (the restatement, see ``behf_oracle.h``) and, where it
was built, ``oracle/_ref/libbehf_ref.so`` (the reference's own kernel bodies on the CPU).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

NFIELD, NMOD, NCOEF = 13, 9, 23
FIELDS = ["vx", "vy", "vz", "qx", "qy", "qz", "sxx", "syy", "szz", "sxy", "sxz", "syz", "p"]
MODULI = ["rho", "rhof", "mu", "M", "C", "HH", "H2u", "C1", "C2"]
PRECISIONS = {"f64": 0, "f32": 1, "f16": 2, "bf16": 3}
SOURCES = {"explosive": 0, "pressure": 1, "force_z": 2}

_P = C.POINTER
_lib = None
_ref = None


class OrcCfg(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("radius", C.c_int),
        ("h", C.c_double), ("dt", C.c_double), ("precision", C.c_int), ("ref_bug_compat", C.c_int),
        ("cpml_width", C.c_int), ("cpml_v0", C.c_double), ("cpml_r", C.c_double),
        ("scale", C.c_double * 4),
        ("src_kind", C.c_int), ("src_ix", C.c_int), ("src_iy", C.c_int), ("src_iz", C.c_int),
        ("src_factor", C.c_double), ("nthreads", C.c_int), ("time_from_step", C.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(_build.build_oracle()))
        _lib.orc_run.restype = C.c_int
        _lib.orc_ref_run.restype = C.c_int
        _lib.orc_ref_aux_name.restype = C.c_char_p
        _lib.orc_last_step_seconds.restype = C.c_double
        _lib.orc_threads.restype = C.c_int
    return _lib


def ref_lib():
    """The reference kernels compiled for the CPU, or None where the reference tree is absent."""
    global _ref
    if _ref is None:
        p = _build.build_ref()
        if p is None:
            return None
        _ref = C.CDLL(str(p))
        _ref.ref_run.restype = C.c_int
        _ref.ref_medium.restype = C.c_int
    return _ref


def _ptrs(arrs, ctype):
    return (_P(ctype) * len(arrs))(*[a.ctypes.data_as(_P(ctype)) for a in arrs])


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ------------------------------------------------------------------------------ medium
def medium_borehole(nz: int, ny: int, nx: int) -> np.ndarray:
    """Restated reference borehole medium, float32 [9, nz, ny, nx]."""
    out = np.zeros((NMOD, nz, ny, nx), np.float32)
    lib().orc_medium_borehole(nz, ny, nx, _ptrs(list(out), C.c_float))
    return out


def ref_medium(nz: int, ny: int, nx: int) -> np.ndarray | None:
    """The reference's own create_model_all, float32 [9, nz, ny, nx]; None without the tree."""
    r = ref_lib()
    if r is None:
        return None
    out = np.zeros((NMOD, nz, ny, nx), np.float32)
    r.ref_medium(nz, ny, nx, _ptrs(list(out), C.c_float))
    return out


def rock_moduli(Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau) -> np.ndarray:
    out = np.zeros(NMOD, np.float64)
    lib().orc_rock_moduli(*[C.c_double(v) for v in (Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau)],
                          out.ctypes.data_as(_P(C.c_double)))
    return out


def build_coeffs(mod: np.ndarray, dt: float) -> np.ndarray:
    _, nz, ny, nx = mod.shape
    mod = _c(mod, np.float32)
    out = np.zeros((NCOEF, nz, ny, nx), np.float64)
    lib().orc_build_coeffs(nx, ny, nz, C.c_double(dt), _ptrs(list(mod), C.c_float), _ptrs(list(out), C.c_double))
    return out


def cpml_profile(n, L, h, dt, v0, rc):
    d, d2, e, e2 = (np.zeros(n) for _ in range(4))
    lib().orc_cpml_profile(n, L, C.c_double(h), C.c_double(dt), C.c_double(v0), C.c_double(rc),
                           *[a.ctypes.data_as(_P(C.c_double)) for a in (d, d2, e, e2)])
    return d, d2, e, e2


def ricker(nt, dt, f0, t0=None, amp=1.0) -> np.ndarray:
    t0 = 1.2 / f0 if t0 is None else t0
    w = np.zeros(nt, np.float32)
    lib().orc_ricker(nt, C.c_double(dt), C.c_double(f0), C.c_double(t0), C.c_double(amp),
                     w.ctypes.data_as(_P(C.c_float)))
    return w


# ------------------------------------------------------------------------------ BEHF run
def run(prob, precision: str = "f64", nthreads: int = 0, nt: int | None = None,
        want_fields: bool = False, time_from_step: int = 0):
    """Oracle run of a problem description (the attributes of behf.problems.Problem).

    Returns (seis [nrec, nt] float64, fields [13, nz, ny, nx] float64 or None)."""
    nt = prob.nt if nt is None else nt
    cfg = OrcCfg()
    cfg.nx, cfg.ny, cfg.nz, cfg.radius = prob.nx, prob.ny, prob.nz, prob.radius
    cfg.h, cfg.dt = prob.h, prob.dt
    cfg.precision = PRECISIONS[precision]
    cfg.ref_bug_compat = int(prob.ref_bug_compat)
    cfg.cpml_width, cfg.cpml_v0, cfg.cpml_r = prob.cpml_width, prob.cpml_v0, prob.cpml_r
    for i in range(4):
        cfg.scale[i] = prob.scales[i]
    cfg.src_kind = SOURCES[prob.src_kind]
    cfg.src_ix, cfg.src_iy, cfg.src_iz = prob.src
    cfg.nthreads = nthreads
    cfg.time_from_step = time_from_step
    mod = _c(prob.mod, np.float32)
    w = _c(prob.wavelet[:nt], np.float32)
    ri = _c(prob.rec_ijk, np.int32).reshape(-1)
    rc = _c(prob.rec_comp, np.int32)
    nrec = rc.shape[0]
    seis = np.zeros((nrec, nt), np.float64)
    fo = np.zeros((NFIELD, prob.nz, prob.ny, prob.nx), np.float64) if want_fields else None
    rcode = lib().orc_run(C.byref(cfg), _ptrs(list(mod), C.c_float), w.ctypes.data_as(_P(C.c_float)), nt, nrec,
                          ri.ctypes.data_as(_P(C.c_int)), rc.ctypes.data_as(_P(C.c_int)),
                          seis.ctypes.data_as(_P(C.c_double)),
                          fo.ctypes.data_as(_P(C.c_double)) if fo is not None else None)
    if rcode != 0:
        raise ValueError(f"orc_run failed with {rcode}")
    return seis, fo


def _cfg(prob, precision="f64", nthreads=0):
    cfg = OrcCfg()
    cfg.nx, cfg.ny, cfg.nz, cfg.radius = prob.nx, prob.ny, prob.nz, prob.radius
    cfg.h, cfg.dt = prob.h, prob.dt
    cfg.precision = PRECISIONS[precision]
    cfg.ref_bug_compat = int(prob.ref_bug_compat)
    cfg.cpml_width, cfg.cpml_v0, cfg.cpml_r = prob.cpml_width, prob.cpml_v0, prob.cpml_r
    for i in range(4):
        cfg.scale[i] = 1.0
    cfg.src_kind = SOURCES[prob.src_kind]
    cfg.src_ix, cfg.src_iy, cfg.src_iz = prob.src
    cfg.nthreads = nthreads
    return cfg


def adjoint(prob, adj_src=None, stride: int = 0, nt: int | None = None, want_coef: bool = False,
            mod=None, nthreads: int = 0, lf_scale=None):
    """FP64 discrete adjoint (behf_adjoint.cpp) of a problem description, physical units.

    adj_src [nrec, nt]: dJ/d seismogram sample (None: zero).  mod overrides prob.mod.  lf_scale [13]: store the
    adjoint state as binary16 times these per-field scales between steps (None: FP64).
    Returns dict(seis [nrec, nt], grad_wavelet [nt], grad_mod [9, nz, ny, nx], grad_coef [23, ...] or None,
    lf_max [13] (largest magnitude of each adjoint field), lf_saturated (values that overflowed binary16))."""
    nt = prob.nt if nt is None else nt
    cfg = _cfg(prob, "f64", nthreads)
    mod = _c(prob.mod if mod is None else mod, np.float32)
    w = _c(prob.wavelet[:nt], np.float32)
    ri = _c(prob.rec_ijk, np.int32).reshape(-1)
    rc = _c(prob.rec_comp, np.int32)
    nrec = rc.shape[0]
    adj = None if adj_src is None else _c(adj_src, np.float64).reshape(nrec, nt)
    seis = np.zeros((nrec, nt), np.float64)
    gw = np.zeros(nt, np.float64)
    gmod = np.zeros((NMOD, prob.nz, prob.ny, prob.nx), np.float64)
    gcoef = np.zeros((NCOEF, prob.nz, prob.ny, prob.nx), np.float64) if want_coef else None
    D = lambda a: a.ctypes.data_as(_P(C.c_double)) if a is not None else None  # noqa: E731
    scale = None if lf_scale is None else _c(lf_scale, np.float64)
    lf_max = np.zeros(NFIELD, np.float64)
    sat = C.c_longlong(0)
    lib().orc_adjoint_ex.restype = C.c_int
    rcode = lib().orc_adjoint_ex(C.byref(cfg), _ptrs(list(mod), C.c_float), w.ctypes.data_as(_P(C.c_float)), nt,
                                 nrec, ri.ctypes.data_as(_P(C.c_int)), rc.ctypes.data_as(_P(C.c_int)), D(adj),
                                 int(stride), D(seis), D(gw), D(gcoef), D(gmod), D(scale), D(lf_max), C.byref(sat))
    if rcode != 0:
        raise ValueError(f"orc_adjoint failed with {rcode}")
    return {"seis": seis, "grad_wavelet": gw, "grad_mod": gmod, "grad_coef": gcoef, "lf_max": lf_max,
            "lf_saturated": int(sat.value)}


def last_step_seconds() -> float:
    """Wall seconds of the time-step loop of the last run() (set-up excluded)."""
    return float(lib().orc_last_step_seconds())


def threads() -> int:
    return int(lib().orc_threads())


# ------------------------------------------------------------------------------ reference mode
def ref_aux_names() -> list[str]:
    return [lib().orc_ref_aux_name(i).decode() for i in range(48)]


def ref_inputs(mod: np.ndarray, h: float, dt: float, np_cells: int, v0: float = 4000.0, rc: float = 1e-6):
    """FP16 coefficient [23,...] and profile [12,...] arrays as main.cpp builds them (uint16 bits)."""
    _, nz, ny, nx = mod.shape
    mod = _c(mod, np.float32)
    coef = np.zeros((NCOEF, nz, ny, nx), np.uint16)
    prof = np.zeros((12, nz, ny, nx), np.uint16)
    lib().orc_ref_inputs(nx, ny, nz, C.c_float(h), C.c_float(dt), np_cells, C.c_float(v0), C.c_float(rc),
                         _ptrs(list(mod), C.c_float), _ptrs(list(coef), C.c_uint16), _ptrs(list(prof), C.c_uint16))
    return coef, prof


def _ref_call(fn, shape, dt, nt, sn, wavelet, state, coef, prof, aux, rec_lin, rec_comp, extra=()):
    nz, ny, nx = shape
    w = _c(wavelet[:nt], np.float32)
    rl = _c(rec_lin, np.int32)
    rcomp = _c(rec_comp, np.int32)
    seis = np.zeros((rl.shape[0], nt), np.float32)
    args = [nx, ny, nz, C.c_float(dt), nt, sn, w.ctypes.data_as(_P(C.c_float)),
            _ptrs(list(state), C.c_uint16), _ptrs(list(coef), C.c_uint16), _ptrs(list(prof), C.c_uint16),
            _ptrs(list(aux), C.c_uint16), rl.shape[0], rl.ctypes.data_as(_P(C.c_int)),
            rcomp.ctypes.data_as(_P(C.c_int)), seis.ctypes.data_as(_P(C.c_float)), *extra]
    rcode = fn(*args)
    if rcode != 0:
        raise ValueError(f"reference-mode run failed with {rcode}")
    return seis


def ref_run(shape, dt, nt, sn, wavelet, state, coef, prof, aux, rec_lin, rec_comp, use_reference=False,
            nthreads=0):
    """Run the reference arithmetic in place on uint16 arrays (state [16,...], aux [48,...]).

    use_reference=False: the oracle's restatement; True: the reference's kernel bodies."""
    for a in (state, coef, prof, aux):
        assert a.dtype == np.uint16 and a.flags.c_contiguous
    if use_reference:
        r = ref_lib()
        if r is None:
            raise RuntimeError("reference tree not available")
        return _ref_call(r.ref_run, shape, dt, nt, sn, wavelet, state, coef, prof, aux, rec_lin, rec_comp)
    return _ref_call(lib().orc_ref_run, shape, dt, nt, sn, wavelet, state, coef, prof, aux, rec_lin, rec_comp,
                     extra=(nthreads,))


def f2h_bits(x: np.ndarray) -> np.ndarray:
    return np.asarray(x, np.float32).astype(np.float16).view(np.uint16)


def h2f(bits: np.ndarray) -> np.ndarray:
    return np.asarray(bits, np.uint16).view(np.float16).astype(np.float32)


def rel_l2(a: np.ndarray, ref: np.ndarray) -> float:
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.linalg.norm(ref.ravel())
    return float(np.linalg.norm((a - ref).ravel()) / den) if den > 0 else float(np.linalg.norm(a.ravel()))


__all__ = [n for n in dir() if not n.startswith("_")]
