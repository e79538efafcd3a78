"""Python front end of libbehf (GB300 BEHF poroelastic time stepper), over its C ABI via ctypes.

The compute path is the CUDA library ``behf/_lib/libbehf.so`` (built by ``behf.build``); this module
only moves host arrays across the C ABI declared in ``include/behf.h``.  There is no CPU fallback:
if the library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

# BEHF_LIBRARY overrides the in-tree build (e.g. to compare builds with different compile-time options).
_LIB_PATH = Path(os.environ.get("BEHF_LIBRARY") or Path(__file__).resolve().parent / "_lib" / "libbehf.so")
_lib = None

FIELDS = ["vx", "vy", "vz", "qx", "qy", "qz", "sxx", "syy", "szz", "sxy", "sxz", "syz", "p"]
FIELD = {n: i for i, n in enumerate(FIELDS)}
MODULI = ["rho", "rhof", "mu", "M", "C", "HH", "H2u", "C1", "C2"]
PHYSICAL = ["lambda", "mu", "rho", "rhof", "M", "alpha", "kappa"]
PRECISION = {"f64": 0, "f32": 1, "f16": 2, "bf16": 3}
SOURCE = {"explosive": 0, "pressure": 1, "force_z": 2}
KERNEL = {"auto": 0, "plain": 1, "tiled": 2}
(OPT_KERNEL, OPT_REF_BUG_COMPAT, OPT_GRAPH_CHUNK, OPT_GRADIENT, OPT_CHECKPOINT, OPT_ZCHUNK, OPT_COEF_ROUNDING,
 OPT_STATE_ROUNDING, OPT_SNAPSHOT_CACHE, OPT_CHECKPOINT_OUTER, OPT_TILED_VARIANT, OPT_GRAD_COMPENSATION,
 OPT_RECOMPUTE_OVERLAP, OPT_TILE_ROWS) = range(14)
TILED_VARIANT = {"auto": 0, "classic": 1, "ws": 2, "tmem": 3, "tmem_xs": 4}
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "allocation failed", -4: "call out of order",
          -5: "non-finite or saturated field", -6: "unsupported"}


class BehfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double), ("dt", C.c_double),
                ("radius", C.c_int), ("cpml_width", C.c_int), ("cpml_v0", C.c_double), ("cpml_r", C.c_double),
                ("scales", C.c_double * 4), ("src_amp_hint", C.c_double), ("src_f0_hint", C.c_double)]


class Rock(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("Ks", "Kf", "Kdry", "mu", "rhos", "rhof", "phi", "kappa", "eta", "tau")]


class MediumSpec(C.Structure):
    _fields_ = [("nlayers", C.c_int), ("layers", Rock * 4), ("interface_z", C.c_int * 3), ("seed", C.c_int),
                ("corr_cells", C.c_double), ("pct", C.c_double), ("log_kappa_sigma", C.c_double),
                ("anomaly", C.c_int), ("anom_center", C.c_double * 3), ("anom_radius_cells", C.c_double),
                ("anom_dkdry", C.c_double), ("anom_kappa_factor", C.c_double)]


def medium_spec(layers, interfaces=(), seed=1234, corr_cells=10.0, pct=0.0, log_kappa_sigma=0.0,
                anomaly=None) -> MediumSpec:
    """C struct of a synthetic medium (same arguments as behf.problems.spec_medium)."""
    s = MediumSpec()
    s.nlayers = len(layers)
    for i, r in enumerate(layers):
        for k, v in r.items():
            setattr(s.layers[i], k, float(v))
    for i, z in enumerate(interfaces):
        s.interface_z[i] = int(z)
    s.seed, s.corr_cells, s.pct, s.log_kappa_sigma = int(seed), float(corr_cells), float(pct), float(log_kappa_sigma)
    if anomaly:
        s.anomaly = 1
        for i in range(3):
            s.anom_center[i] = float(anomaly["center"][i])
        s.anom_radius_cells = float(anomaly["radius"])
        s.anom_dkdry = float(anomaly["dkdry"])
        s.anom_kappa_factor = float(anomaly["kappa_factor"])
    return s


class Info(C.Structure):
    _fields_ = [("step", C.c_int64), ("device_bytes", C.c_int64), ("scales", C.c_double * 4),
                ("bytes_per_cell", C.c_double), ("kernel", C.c_int), ("radius", C.c_int), ("precision", C.c_int),
                ("launches", C.c_int64), ("tiled_variant", C.c_int), ("zchunk", C.c_int), ("tile_rows", C.c_int)]


def lib_path() -> Path:
    return _LIB_PATH


def load() -> C.CDLL:
    """Load libbehf.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise RuntimeError(f"{_LIB_PATH} is missing: build it with behf.build.build()")
    lib = C.CDLL(str(_LIB_PATH))
    P = C.POINTER
    sig = {
        "behf_create": [P(Grid), C.c_int, P(C.c_void_p)],
        "behf_destroy": [C.c_void_p],
        "behf_set_medium": [C.c_void_p, P(P(C.c_float))],
        "behf_set_medium_device": [C.c_void_p, P(C.c_void_p)],
        "behf_generate_medium": [C.c_void_p, P(MediumSpec)],
        "behf_set_cpml_profile": [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double)],
        "behf_set_source": [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_float), C.c_int],
        "behf_set_receivers": [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int), C.c_int],
        "behf_run": [C.c_void_p, C.c_int],
        "behf_run_async": [C.c_void_p, C.c_int],
        "behf_sync": [C.c_void_p],
        "behf_get_seismograms": [C.c_void_p, P(C.c_double), P(C.c_int)],
        "behf_get_field": [C.c_void_p, C.c_int, P(C.c_float)],
        "behf_set_field": [C.c_void_p, C.c_int, P(C.c_float)],
        "behf_reset": [C.c_void_p],
        "behf_set_option": [C.c_void_p, C.c_int, C.c_int],
        "behf_get_info": [C.c_void_p, P(Info)],
        "behf_get_stream": [C.c_void_p, P(C.c_void_p)],
        "behf_health": [C.c_void_p, P(C.c_double)],
        "behf_update_wavelet": [C.c_void_p, C.c_int, P(C.c_float), C.c_int],
        "behf_get_seismograms_range": [C.c_void_p, C.c_int, C.c_int, P(C.c_double)],
        "behf_time_kernels": [C.c_void_p, C.c_int, P(C.c_double)],
        "behf_gradient": [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double), P(P(C.c_double))],
        "behf_misfit_gradient": [C.c_void_p, C.c_int, P(C.c_double), P(C.c_double), P(C.c_double),
                                 P(P(C.c_double))],
        "behf_autotune": [C.c_void_p, C.c_int, P(C.c_int), P(C.c_double)],
        "behf_selftest_wait": [C.c_void_p],
        "behf_run_batch": [P(C.c_void_p), C.c_int, C.c_int],
        "behf_checkpoint_plan": [C.c_int, C.c_int, C.c_int, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t,
                                 P(C.c_int), P(C.c_int), P(C.c_size_t)],
        "behf_field_norm_noalloc": [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_longlong,
                                    C.c_void_p, C.c_void_p, C.c_void_p],
        "behf_physical_gradient": [C.c_longlong, P(P(C.c_float)), P(P(C.c_double)), C.c_double, P(P(C.c_double))],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.behf_last_error.restype = C.c_char_p
    lib.behf_last_error.argtypes = []
    lib.behf_version.restype = C.c_char_p
    _lib = lib
    return lib


def _check(code: int):
    if code != 0:
        raise BehfError(code, load().behf_last_error().decode())


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Solver:
    """One BEHF context on the current CUDA device (owns its stream and device memory)."""

    def __init__(self, nx, ny, nz, h, dt, radius=4, precision="f16", cpml_width=10, cpml_v0=4000.0,
                 cpml_r=1e-6, scales=None, src_amp_hint=0.0, src_f0_hint=0.0):
        self._lib = load()
        g = Grid()
        g.nx, g.ny, g.nz, g.h, g.dt, g.radius = nx, ny, nz, h, dt, radius
        g.cpml_width, g.cpml_v0, g.cpml_r = cpml_width, cpml_v0, cpml_r
        for i in range(4):
            g.scales[i] = 0.0 if scales is None else float(scales[i])
        g.src_amp_hint, g.src_f0_hint = src_amp_hint, src_f0_hint
        self.grid = g
        self.shape = (nz, ny, nx)
        self.precision = precision
        self._ctx = C.c_void_p()
        _check(self._lib.behf_create(C.byref(g), PRECISION[precision], C.byref(self._ctx)))
        self.nrec = 0

    # -- lifecycle
    def close(self):
        if self._ctx:
            self._lib.behf_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- set-up
    def set_medium(self, mod: np.ndarray):
        mod = _f32(mod)
        assert mod.shape == (9, *self.shape), mod.shape
        ptrs = (C.POINTER(C.c_float) * 9)(*[mod[i].ctypes.data_as(C.POINTER(C.c_float)) for i in range(9)])
        _check(self._lib.behf_set_medium(self._ctx, ptrs))

    def set_medium_device(self, ptrs: list[int]):
        arr = (C.c_void_p * 9)(*ptrs)
        _check(self._lib.behf_set_medium_device(self._ctx, arr))

    def generate_medium(self, spec: dict):
        """Device-side synthetic medium (spec: the arguments of behf.problems.spec_medium)."""
        cs = medium_spec(**spec)
        _check(self._lib.behf_generate_medium(self._ctx, C.byref(cs)))

    def set_cpml_profile(self, axis: int, d: np.ndarray, d2: np.ndarray):
        d = np.ascontiguousarray(d, np.float64)
        d2 = np.ascontiguousarray(d2, np.float64)
        _check(self._lib.behf_set_cpml_profile(self._ctx, axis, d.ctypes.data_as(C.POINTER(C.c_double)),
                                               d2.ctypes.data_as(C.POINTER(C.c_double))))

    def set_source(self, kind: str, ijk, wavelet: np.ndarray):
        w = _f32(wavelet)
        _check(self._lib.behf_set_source(self._ctx, SOURCE[kind], int(ijk[0]), int(ijk[1]), int(ijk[2]),
                                         w.ctypes.data_as(C.POINTER(C.c_float)), int(w.shape[0])))

    def set_receivers(self, ijk: np.ndarray, comp: np.ndarray, capacity: int):
        ijk = np.ascontiguousarray(ijk, np.int32).reshape(-1, 3)
        comp = np.ascontiguousarray(comp, np.int32)
        self.nrec = comp.shape[0]
        _check(self._lib.behf_set_receivers(self._ctx, self.nrec, ijk.ctypes.data_as(C.POINTER(C.c_int)),
                                            comp.ctypes.data_as(C.POINTER(C.c_int)), int(capacity)))

    def set_option(self, opt: int, value: int):
        _check(self._lib.behf_set_option(self._ctx, opt, int(value)))

    def set_kernel(self, name: str):
        self.set_option(OPT_KERNEL, KERNEL[name])

    # -- running
    def run(self, nsteps: int):
        _check(self._lib.behf_run(self._ctx, int(nsteps)))

    def run_async(self, nsteps: int):
        _check(self._lib.behf_run_async(self._ctx, int(nsteps)))

    def sync(self):
        _check(self._lib.behf_sync(self._ctx))

    def reset(self):
        _check(self._lib.behf_reset(self._ctx))

    # -- outputs
    def seismograms(self) -> np.ndarray:
        ns = C.c_int(0)
        _check(self._lib.behf_get_seismograms(self._ctx, None, C.byref(ns)))
        out = np.zeros((self.nrec, ns.value), np.float64)
        if self.nrec and ns.value:
            _check(self._lib.behf_get_seismograms(self._ctx, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                  C.byref(ns)))
        return out

    def get_field(self, name) -> np.ndarray:
        q = FIELD[name] if isinstance(name, str) else int(name)
        out = np.zeros(self.shape, np.float32)
        _check(self._lib.behf_get_field(self._ctx, q, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_field(self, name, values: np.ndarray):
        q = FIELD[name] if isinstance(name, str) else int(name)
        v = _f32(values)
        assert v.shape == self.shape
        _check(self._lib.behf_set_field(self._ctx, q, v.ctypes.data_as(C.POINTER(C.c_float))))

    def info(self) -> dict:
        inf = Info()
        _check(self._lib.behf_get_info(self._ctx, C.byref(inf)))
        return {"step": inf.step, "device_bytes": inf.device_bytes, "scales": tuple(inf.scales),
                "bytes_per_cell": inf.bytes_per_cell, "kernel": {0: "auto", 1: "plain", 2: "tiled"}[inf.kernel],
                "radius": inf.radius, "precision": inf.precision, "launches": inf.launches,
                "tiled_variant": {1: "classic", 2: "ws", 3: "tmem", 4: "tmem_xs"}.get(inf.tiled_variant, "classic"),
                "zchunk": inf.zchunk, "tile_rows": inf.tile_rows}

    def update_wavelet(self, it0: int, w: np.ndarray):
        w = _f32(w)
        _check(self._lib.behf_update_wavelet(self._ctx, int(it0), w.ctypes.data_as(C.POINTER(C.c_float)),
                                             int(w.shape[0])))

    def seismograms_range(self, it0: int, n: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros((self.nrec, n), np.float64)
        _check(self._lib.behf_get_seismograms_range(self._ctx, int(it0), int(n),
                                                    out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def time_kernels(self, nsteps: int) -> dict:
        ms = np.zeros(4, np.float64)
        _check(self._lib.behf_time_kernels(self._ctx, int(nsteps), ms.ctypes.data_as(C.POINTER(C.c_double))))
        return {"source": ms[0], "velocity": ms[1], "stress": ms[2], "record": ms[3]}

    def autotune(self, trial_steps: int = 4):
        """Pick the fastest tile height, tiled-kernel variant and z-chunk length; resets the wavefields.  Returns
        (zchunk, ms/step); the variant and height are info()["tiled_variant"] and info()["tile_rows"]."""
        z, ms = C.c_int(0), C.c_double(0)
        _check(self._lib.behf_autotune(self._ctx, int(trial_steps), C.byref(z), C.byref(ms)))
        return z.value, ms.value

    def selftest_wait(self) -> int:
        """Failure-detection self-test: a bounded pipeline wait that nothing releases (about 2 s); returns the
        status code, BEHF_ERR_TIMEOUT (-7) when detection works.  The context stays usable."""
        return int(self._lib.behf_selftest_wait(self._ctx))

    # -- gradient (adjoint state, checkpointed)
    def enable_gradient(self, checkpoint: int = 0, snapshot_cache: int = -1, checkpoint_outer: int = 0,
                        overlap: int = 1):
        """Keep the moduli on the device for behf_gradient (call before the medium); checkpoint = steps
        between checkpoints of the gradient's forward pass (0 = round(sqrt(nt))); snapshot_cache = device MiB
        for keeping the forward pass's snapshots of the last segments (-1 automatic, 0 none: every segment is
        recomputed from its checkpoint); checkpoint_outer = outer spacing of the two-level scheme (0 automatic:
        two levels only when one does not fit the device memory); overlap = 1: a segment's recompute runs on a
        second stream while the previous segment's adjoint steps run (0: one after the other)."""
        self.set_option(OPT_GRADIENT, 1)
        self.set_option(OPT_CHECKPOINT, int(checkpoint))
        self.set_option(OPT_SNAPSHOT_CACHE, int(snapshot_cache))
        self.set_option(OPT_CHECKPOINT_OUTER, int(checkpoint_outer))
        self.set_option(OPT_RECOMPUTE_OVERLAP, int(overlap))

    def _grad_out(self, nt, moduli):
        gw = np.zeros(nt, np.float64)
        gm = np.zeros((9,) + self.shape, np.float64) if moduli else None
        arr = (C.POINTER(C.c_double) * 9)(*[gm[q].ctypes.data_as(C.POINTER(C.c_double)) if moduli else None
                                            for q in range(9)])
        return gw, gm, arr

    def gradient(self, nt: int, adj_src: np.ndarray, moduli: bool = True):
        """Adjoint-state gradient for the adjoint source adj_src [nrec, nt] (dJ/d seismogram, physical units).
        Returns (dJ/d wavelet [nt], dJ/d moduli [9, nz, ny, nx] or None)."""
        adj = np.ascontiguousarray(adj_src, np.float64).reshape(self.nrec, nt)
        gw, gm, arr = self._grad_out(nt, moduli)
        _check(self._lib.behf_gradient(self._ctx, int(nt), adj.ctypes.data_as(C.POINTER(C.c_double)),
                                       gw.ctypes.data_as(C.POINTER(C.c_double)), arr))
        return gw, gm

    def misfit_gradient(self, nt: int, observed: np.ndarray, moduli: bool = True):
        """L2 misfit J = 1/2 |seis - observed|^2 and its gradient.  Returns (J, dJ/d wavelet, dJ/d moduli)."""
        obs = np.ascontiguousarray(observed, np.float64).reshape(self.nrec, nt)
        gw, gm, arr = self._grad_out(nt, moduli)
        J = C.c_double(0)
        _check(self._lib.behf_misfit_gradient(self._ctx, int(nt), obs.ctypes.data_as(C.POINTER(C.c_double)),
                                              C.byref(J), gw.ctypes.data_as(C.POINTER(C.c_double)), arr))
        return J.value, gw, gm

    def health(self):
        norms = np.zeros(13, np.float64)
        code = self._lib.behf_health(self._ctx, norms.ctypes.data_as(C.POINTER(C.c_double)))
        if code not in (0, -5):
            _check(code)
        return code == 0, norms

    def stream(self) -> int:
        s = C.c_void_p()
        _check(self._lib.behf_get_stream(self._ctx, C.byref(s)))
        return s.value or 0


def field_norm_noalloc(field_ptr: int, precision: str, nx: int, ny: int, nz: int, pitch: int, plane: int,
                       norm_ptr: int, flag_ptr: int, stream: int = 0):
    """behf_field_norm_noalloc on caller-owned device pointers (see include/behf.h): the energy norm and
    health flag of one field without any device allocation.  Asynchronous on `stream`."""
    _check(load().behf_field_norm_noalloc(C.c_void_p(field_ptr), PRECISION[precision], nx, ny, nz, pitch, plane,
                                          C.c_void_p(norm_ptr), C.c_void_p(flag_ptr), C.c_void_p(stream)))


def physical_gradient(mod: np.ndarray, grad_mod: np.ndarray, eta: float = 1e-3) -> np.ndarray:
    """behf_physical_gradient (host, no GPU): dJ/d(lambda, mu, rho, rho_f, M, alpha, kappa) [7, ...] from the
    moduli [9, ...] of the medium and the moduli gradient [9, ...] of Solver.gradient / misfit_gradient."""
    mod = np.ascontiguousarray(mod, dtype=np.float32)
    gm = np.ascontiguousarray(grad_mod, dtype=np.float64)
    if mod.shape[0] != 9 or gm.shape != mod.shape:
        raise ValueError("moduli and their gradient must both be [9, ...] of one shape")
    n = int(np.prod(mod.shape[1:]))
    out = np.zeros((7, *mod.shape[1:]), np.float64)
    mp = (C.POINTER(C.c_float) * 9)(*[mod[q].ctypes.data_as(C.POINTER(C.c_float)) for q in range(9)])
    gp = (C.POINTER(C.c_double) * 9)(*[gm[q].ctypes.data_as(C.POINTER(C.c_double)) for q in range(9)])
    op = (C.POINTER(C.c_double) * 7)(*[out[q].ctypes.data_as(C.POINTER(C.c_double)) for q in range(7)])
    _check(load().behf_physical_gradient(n, mp, gp, float(eta), op))
    return out


def algorithmic_bytes(precision: str, shape, cpml_width: int) -> dict:
    """Compulsory HBM bytes per cell update of each kernel and of a whole step.

    velocity: reads 7 stresses/pressure + 6 v/q, writes 6 v/q; 3 FP32 Darcy factors + 12 coefficients;
              CPML psi + previous derivative (FP32) read and written for its 4 derivatives per axis on
              the slab fraction W/n of that axis (W = 2L+1).
    stress:   reads 6 v/q + 7 stresses/pressure, writes 7; 8 coefficients; CPML as velocity.
    step_fused: the per-step figure with each field read and written once (26 field accesses),
              23 coefficients and the CPML memory -- the algorithmic bytes of one cell update."""
    es = {"f64": 8, "f32": 4, "f16": 2, "bf16": 2}[precision]
    ks = {"f64": 8, "f32": 4, "f16": 2, "bf16": 2}[precision]
    ws = 8 if precision == "f64" else 4
    W = 2 * cpml_width + 1 if cpml_width > 0 else 0
    cpml_half = sum(4 * 2 * 2 * ws * W / n for n in shape)
    vel = 19 * es + 3 * ws + 12 * ks + cpml_half
    strs = 20 * es + 8 * ks + cpml_half
    fused = 26 * es + 3 * ws + 20 * ks + 2 * cpml_half
    return {"velocity": vel, "stress": strs, "step_unfused": vel + strs, "step_fused": fused}


def checkpoint_plan(nt: int, ck_bytes: int, snap_bytes: int, avail: int, checkpoint: int = 0,
                    checkpoint_outer: int = 0, fixed_bytes: int = 0) -> tuple[int, int, int]:
    """The gradient's checkpoint plan (behf_checkpoint_plan; no GPU needed): (inner spacing, outer spacing, device
    bytes); outer == inner means one level."""
    inner, outer, nbytes = C.c_int(), C.c_int(), C.c_size_t()
    _check(load().behf_checkpoint_plan(int(nt), int(checkpoint), int(checkpoint_outer), int(ck_bytes),
                                       int(snap_bytes), int(fixed_bytes), int(avail), C.byref(inner),
                                       C.byref(outer), C.byref(nbytes)))
    return inner.value, outer.value, nbytes.value


def run_batch(solvers, nsteps: int):
    """Advance independent solvers (shots) together on the device: their streams overlap."""
    arr = (C.c_void_p * len(solvers))(*[s._ctx.value for s in solvers])
    _check(load().behf_run_batch(arr, len(solvers), int(nsteps)))


def solver_for(prob, precision="f16", kernel="auto", scales=None, capacity=None, gradient=False,
               checkpoint=0, coef_rounding=0, state_rounding=0, snapshot_cache=-1, checkpoint_outer=0,
               overlap=1) -> Solver:
    """A Solver set up with a problem description (see behf.problems.Problem); gradient=True keeps what
    Solver.gradient needs."""
    s = Solver(prob.nx, prob.ny, prob.nz, prob.h, prob.dt, radius=prob.radius, precision=precision,
               cpml_width=prob.cpml_width, cpml_v0=prob.cpml_v0, cpml_r=prob.cpml_r, scales=scales,
               src_amp_hint=float(np.abs(prob.wavelet).max()) if prob.wavelet.size else 1.0,
               src_f0_hint=prob.f0)
    if prob.ref_bug_compat:
        s.set_option(OPT_REF_BUG_COMPAT, 1)
    s.set_kernel(kernel)
    if gradient:
        s.enable_gradient(checkpoint, snapshot_cache, checkpoint_outer, overlap)
    if coef_rounding:
        s.set_option(OPT_COEF_ROUNDING, int(coef_rounding))
    if state_rounding:
        s.set_option(OPT_STATE_ROUNDING, int(state_rounding))
    if prob.mod.shape[1:] == (prob.nz, prob.ny, prob.nx):
        s.set_medium(prob.mod)
    else:
        s.generate_medium(prob.extra["spec"])
    s.set_source(prob.src_kind, prob.src, prob.wavelet)
    if len(prob.rec_comp):
        s.set_receivers(prob.rec_ijk, prob.rec_comp, prob.nt if capacity is None else capacity)
    return s


__all__ = ["Solver", "BehfError", "solver_for", "run_batch", "checkpoint_plan", "physical_gradient", "load", "lib_path",
           "FIELDS", "FIELD", "MODULI", "PHYSICAL"]
