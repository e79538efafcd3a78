"""Problem descriptions: media, sources, receivers and the named workloads.

A ``Problem`` carries everything one forward run needs (grid, cell-centred moduli, wavelet, source,
receivers, CPML) so that the same description drives the CUDA library and the CPU oracle.

Media restate the reference's Biot-Gassmann relations (outputfunc.cpp:202-217):
    rho = (1-phi) rho_s + phi rho_f,  alpha = 1 - K_dry/K_s,
    M = K_f K_s / (phi K_s + (alpha - phi) K_f),  H = alpha^2 M + K_dry + 4 mu / 3,
    lambda_u = H - 2 mu,  C = alpha M,  b = eta / kappa,  m = (1 + 2/8) tau rho_f / phi
(the shape factor 8 is the reference's ``porousm``, outputfunc.cpp:164).  A cell with phi = 1 is pure
fluid, as the reference's borehole cells (outputfunc.cpp:169-187).

Named workloads (sizes, steps and media of the benchmark and parity cases):
    small64       64^3, h = 5 m, dt = 0.4 ms, 500 steps, 10-cell CPML, homogeneous sandstone,
                  explosive source at the centre, 30 Hz Ricker, 32 receivers on a line (vz and p)
    layered256    256^3, 2000 steps, 20-cell CPML, sandstone over a stiffer layer at z = 640 m,
                  25 Hz explosive (pressure) source, 16 x 16 surface receivers (vz and p).  The source is the
                  isotropic-stress "explosive (pressure)" source of small64 and of the reference (kernel.cu:130-142),
                  not an injection into the pore pressure: in this medium a pore-pressure injection radiates a fast
                  wave 1e-4 to 1e-5 of the near-source pressure, which FP32 storage already resolves only to
                  1.7e-3 (oracle, 64^3) and FP16 storage not at all
    random1024    1024^3, 3000 steps, 20-cell CPML, sandstone with 5 % Gaussian-correlated (50 m)
                  perturbations of K_dry, mu, phi and log-normal kappa (sigma 0.5), vertical force
                  source, 20 Hz, 512 x 512 surface receivers (vz and p)
    inversion256  the gradient workload: layered256's medium (+ a 100 m Gaussian anomaly for the true model),
                  16 explosive (pressure) source shots at 25 Hz, 2000 steps, 16 x 16 surface receivers (vz and p)
    borehole      the reference's own problem: 240 x 240 x 360 cells of 1 cm (180^2 x 300 + 30-cell
                  CPML), fluid borehole in a porous formation, 10 kHz, 3500 steps of 1 us, radius 1,
                  txx recorded on the vertical line through the source (main.cpp:20-23, 84-99)
Each accepts a ``scale`` (grid shrink factor) and ``nt`` override for test-sized variants.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SANDSTONE = dict(Ks=37e9, Kf=2.25e9, Kdry=9e9, mu=7e9, rhos=2650.0, rhof=1000.0, phi=0.2, kappa=1e-12,
                 eta=1e-3, tau=2.4)
STIFF = dict(SANDSTONE, Kdry=20e9, mu=15e9, phi=0.1, kappa=1e-14)


def rock_moduli(Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau):
    """Cell-centred moduli [9, ...] (rho, rhof, mu, M, C, HH, H2u, C1, C2) from rock parameters (arrays ok)."""
    Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau = np.broadcast_arrays(
        *[np.asarray(v, np.float64) for v in (Ks, Kf, Kdry, mu, rhos, rhof, phi, kappa, eta, tau)])
    porousm = 8.0
    rho = (1 - phi) * rhos + phi * rhof
    a = 1 - Kdry / Ks
    M = Kf * Ks / (phi * Ks + (a - phi) * Kf)
    HH = a * a * M + Kdry + mu * 4.0 / 3.0
    out = np.stack([rho, rhof, mu, M, M * a, HH, HH - 2 * mu, eta / kappa, (1 + 2 / porousm) * tau * rhof / phi])
    fluid = phi >= 1.0
    if np.any(fluid):
        out[0][fluid] = rhof[fluid]
        out[2][fluid] = 0.0
        for q in (3, 4, 5, 6):
            out[q][fluid] = Kf[fluid]
        out[7][fluid] = 0.0
        out[8][fluid] = rhof[fluid]
    return out


def physical_from_moduli(mod: np.ndarray, eta: float = 1e-3) -> tuple[np.ndarray, np.ndarray]:
    """Biot's physical parameters [7, ...] (lambda, mu, rho, rho_f, M, alpha, kappa) of cell-centred moduli, and the
    per-cell ratio m / rho_f = (1 + 2/8) tau / phi that they leave fixed (the inverse of moduli_from_physical).
    Pure-fluid cells (b = 0) get kappa = inf."""
    m = np.asarray(mod, np.float64)
    rho, rhof, mu, M, Cc, HH, H2u, b, mm = m
    alpha = np.divide(Cc, M, out=np.zeros_like(M), where=M != 0)
    lam = H2u - alpha * alpha * M
    with np.errstate(divide="ignore"):
        kappa = np.where(b > 0, eta / np.where(b > 0, b, 1.0), np.inf)
    ratio = np.divide(mm, rhof, out=np.zeros_like(mm), where=rhof != 0)
    return np.stack([lam, mu, rho, rhof, M, alpha, kappa]), ratio


def moduli_from_physical(phys: np.ndarray, m_over_rhof: np.ndarray, eta: float = 1e-3) -> np.ndarray:
    """Cell-centred moduli [9, ...] float32 from physical parameters [7, ...]: C = alpha M, lambda_u = lambda +
    alpha^2 M, H = lambda_u + 2 mu, b = eta / kappa, m = (m / rho_f) rho_f (outputfunc.cpp:202-217)."""
    lam, mu, rho, rhof, M, alpha, kappa = np.asarray(phys, np.float64)
    h2u = lam + alpha * alpha * M
    b = np.where(np.isfinite(kappa), eta / kappa, 0.0)
    return np.stack([rho, rhof, mu, M, alpha * M, h2u + 2 * mu, h2u, b, m_over_rhof * rhof]).astype(np.float32)


def p_velocity(rock: dict) -> float:
    m = rock_moduli(**rock)
    return float(np.sqrt(m[5] / m[0]))


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = x + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def hash_noise(n_cells: int, f: int, seed: int) -> np.ndarray:
    """Standard normal samples, one per cell: Box-Muller (FP64) on two 24-bit fields of
    splitmix64(cell | f << 32 | seed << 36); the device generator draws the same numbers."""
    c = np.arange(n_cells, dtype=np.uint64) | (np.uint64(f) << np.uint64(32)) | (np.uint64(seed) << np.uint64(36))
    with np.errstate(over="ignore"):
        h = _splitmix64(c)
    u1 = ((h >> np.uint64(40)).astype(np.float64) + 0.5) / 16777216.0
    u2 = (((h >> np.uint64(16)) & np.uint64(0xFFFFFF)).astype(np.float64) + 0.5) / 16777216.0
    return (np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)).astype(np.float32)


def gaussian_weights(corr_cells: float):
    sig = corr_cells / 2.0
    half = int(np.ceil(4 * sig))
    x = np.arange(-half, half + 1)
    g = np.exp(-0.5 * (x / sig) ** 2)
    g /= g.sum()
    return x, g


def gaussian_random_field(shape, corr_cells: float, seed: int, f: int = 0) -> np.ndarray:
    """Zero-mean, unit-variance field with correlation exp(-r^2 / l^2), l = corr_cells.

    Hash noise smoothed by a separable Gaussian of std l/2 (periodic wrap, x then y then z, float32
    accumulation), normalised by the filter's gain (sum w^2)^(3/2) -- the device generator's
    algorithm (kernels_medium.cu)."""
    n = int(np.prod(shape))
    f32 = hash_noise(n, f, seed).reshape(shape)
    x, g = gaussian_weights(corr_cells)
    w = g.astype(np.float32)
    for ax in (2, 1, 0):  # x, y, z of a [z][y][x] array
        acc = np.zeros_like(f32)
        for k, wk in zip(x, w):
            acc += wk * np.roll(f32, int(k), axis=ax)
        f32 = acc
    return f32.astype(np.float64) * (1.0 / np.sqrt(np.sum(g * g)) ** 3)


def spec_medium(shape, layers, interfaces=(), seed=1234, corr_cells=10.0, pct=0.0, log_kappa_sigma=0.0,
                anomaly=None) -> np.ndarray:
    """Host mirror of behf_generate_medium: layered rocks, correlated perturbations, Gaussian anomaly.

    anomaly = dict(center=(x, y, z), radius=R_cells, dkdry=..., kappa_factor=...)."""
    nz, ny, nx = shape
    kk = np.arange(nz)[:, None, None] * np.ones((1, ny, nx))
    layer = np.zeros(shape, np.int64)
    for zi in interfaces:
        layer += (kk >= zi)
    keys = ("Ks", "Kf", "Kdry", "mu", "rhos", "rhof", "phi", "kappa", "eta", "tau")
    par = {k: np.asarray([r[k] for r in layers], np.float64)[layer] for k in keys}
    if pct != 0 or log_kappa_sigma != 0:
        g = [gaussian_random_field(shape, corr_cells, seed, f) for f in range(4)]
        par["Kdry"] = par["Kdry"] * (1 + pct * g[0])
        par["mu"] = par["mu"] * (1 + pct * g[1])
        par["phi"] = np.where(par["phi"] < 1.0, par["phi"] * (1 + pct * g[2]), par["phi"])
        par["kappa"] = par["kappa"] * np.exp(log_kappa_sigma * g[3])
    if anomaly:
        ii = np.arange(nx)[None, None, :]
        jj = np.arange(ny)[None, :, None]
        cx, cy, cz = anomaly["center"]
        G = np.exp(-((ii - cx) ** 2 + (jj - cy) ** 2 + (kk - cz) ** 2) / anomaly["radius"] ** 2)
        par["Kdry"] = par["Kdry"] * (1 + anomaly["dkdry"] * G)
        par["kappa"] = par["kappa"] * np.power(anomaly["kappa_factor"], G)
    return rock_moduli(**par).astype(np.float32)


@dataclass
class Problem:
    nx: int
    ny: int
    nz: int
    h: float
    dt: float
    radius: int
    mod: np.ndarray                  # float32 [9, nz, ny, nx]
    wavelet: np.ndarray              # float32 [nt]
    src: tuple
    rec_ijk: np.ndarray              # int32 [nrec, 3]  (ix, iy, iz)
    rec_comp: np.ndarray             # int32 [nrec]
    src_kind: str = "explosive"
    cpml_width: int = 10
    cpml_v0: float = 4000.0
    cpml_r: float = 1e-6
    f0: float = 30.0
    ref_bug_compat: bool = False
    scales: tuple = (1.0, 1.0, 1.0, 1.0)
    name: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def nt(self) -> int:
        return int(self.wavelet.shape[0])

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz


def auto_scales(mod: np.ndarray, amp: float = 1.0, f0: float = 30.0) -> tuple:
    """The library's automatic storage scales (powers of two), from the moduli and the wavelet:
    s_sigma = s_p = 16/amp, s_v = s_sigma * max sqrt(rho H) (fast-P impedance), and
    s_q = s_v * clamp(b_min / (rho_max 2 pi f0), 1, 1e6) so the Darcy flux, which is smaller than v by
    about rho omega / b at low frequency, lands in the same range."""
    rho = np.maximum(mod[0].astype(np.float64), 0)
    hh = np.maximum(mod[5].astype(np.float64), 0)
    c1 = mod[7].astype(np.float64)
    zmax = float(np.sqrt(rho * hh).max())
    rmax = float(rho.max())
    pos = c1[c1 > 0]
    ss = 16.0 / amp
    sv = ss * (zmax if zmax > 0 else 1.0)
    kq = float(pos.min()) / (rmax * 2 * np.pi * f0) if pos.size and rmax > 0 else 1.0
    kq = min(max(kq, 1.0), 1e6)
    p2 = lambda v: float(2.0 ** round(np.log2(v)))
    return (p2(sv), p2(sv * kq), p2(ss), p2(ss))


def ricker(nt: int, dt: float, f0: float, t0: float | None = None, amp: float = 1.0) -> np.ndarray:
    """Ricker wavelet of kernel.cu:1898: amp * -(1 - 2 pi^2 f^2 tau^2) exp(-pi^2 f^2 tau^2), tau = t - t0,
    t0 = 1.2/f by default (kernel.cu:1730)."""
    t0 = 1.2 / f0 if t0 is None else t0
    tau = np.arange(nt) * dt - t0
    a = (np.pi * f0 * tau) ** 2
    return (amp * -(1 - 2 * a) * np.exp(-a)).astype(np.float32)


def ricker_reference(nt: int, dt: float, f0: float) -> np.ndarray:
    """The same wavelet evaluated as kernel.cu:1890-1898 does: t = it*DT and T0 = 1.2/F0 in float, the
    product in double with pi = 3.1415926535, the result rounded to float."""
    f32 = np.float32
    DT, F0 = f32(dt), f32(f0)
    T0 = f32(1.2 / float(F0))
    pi = 3.1415926535
    w = np.empty(nt, np.float32)
    for it in range(nt):
        d = float(f32(f32(it) * DT) - T0)
        a2 = 2 * pi * pi * float(F0) * float(F0) * d * d
        a = pi * pi * float(F0) * float(F0) * d * d
        w[it] = f32(-(1 - a2) * np.exp(-a))
    return w


def homogeneous(shape, rock=SANDSTONE) -> np.ndarray:
    m = rock_moduli(**rock)
    return np.broadcast_to(m[:, None, None, None], (9, *shape)).astype(np.float32)


def layered(shape, rocks, interfaces) -> np.ndarray:
    """Layers in z: rocks[0] above interfaces[0] (cell index), rocks[1] below, ..."""
    nz = shape[0]
    out = np.empty((9, *shape), np.float32)
    bounds = [0, *interfaces, nz]
    for r, (z0, z1) in zip(rocks, zip(bounds[:-1], bounds[1:])):
        out[:, z0:z1] = rock_moduli(**r)[:, None, None, None]
    return out


def random_medium(shape, rock=SANDSTONE, seed=1234, corr_cells=10.0, pct=0.05, log_kappa_sigma=0.5):
    return spec_medium(shape, [rock], (), seed, corr_cells, pct, log_kappa_sigma)


def random_spec(rock=SANDSTONE, seed=1234, corr_cells=10.0, pct=0.05, log_kappa_sigma=0.5) -> dict:
    """The random1024 medium as a device-generator spec (see behf.Solver.generate_medium)."""
    return dict(layers=[rock], interfaces=(), seed=seed, corr_cells=corr_cells, pct=pct,
                log_kappa_sigma=log_kappa_sigma, anomaly=None)


def line_receivers(ix, iy, iz, comps):
    ix, iy, iz = np.broadcast_arrays(np.atleast_1d(ix), np.atleast_1d(iy), np.atleast_1d(iz))
    ijk = np.stack([ix, iy, iz], 1).astype(np.int32)
    ijk = np.repeat(ijk, len(comps), axis=0)
    comp = np.tile(np.asarray(comps, np.int32), len(ix))
    return ijk, comp


def small64(n=64, nt=500, radius=4, cpml=10) -> Problem:
    h, dt, f0 = 5.0, 4e-4, 30.0
    shape = (n, n, n)
    c = n // 2
    xs = np.linspace(cpml + 2, n - cpml - 3, 32).round().astype(int)
    ijk, comp = line_receivers(xs, c, min(c + 10, n - cpml - 2), [2, 12])
    return Problem(n, n, n, h, dt, radius, homogeneous(shape), ricker(nt, dt, f0), (c, c, c), ijk, comp,
                   cpml_width=cpml, cpml_v0=p_velocity(SANDSTONE), f0=f0, name=f"small{n}")


def layered256(n=256, nt=2000, radius=4, cpml=20, nrec_side=16) -> Problem:
    h, dt, f0 = 5.0, 4e-4, 25.0
    shape = (n, n, n)
    zi = n // 2  # z = 640 m at 256 cells of 5 m
    mod = layered(shape, [SANDSTONE, STIFF], [zi])
    c = n // 2
    ax = np.linspace(cpml + 4, n - cpml - 5, nrec_side).round().astype(int)
    X, Y = np.meshgrid(ax, ax, indexing="xy")
    ijk, comp = line_receivers(X.ravel(), Y.ravel(), cpml + 2, [2, 12])
    src = (c, c, max(cpml + 6, (cpml + zi) // 2))
    return Problem(n, n, n, h, dt, radius, mod, ricker(nt, dt, f0), src, ijk, comp, cpml_width=cpml,
                   cpml_v0=p_velocity(STIFF), f0=f0, name=f"layered{n}")


def inversion256(n=256, nt=2000, shot=0, true_model=True, radius=4, cpml=20, nrec_side=16) -> Problem:
    """The gradient workload: the two-layer 256^3 medium of layered256 (interface at z = 640 m), for the true
    model with a Gaussian anomaly of 100 m radius (K_dry -10 %, kappa x10) above the interface; 25 Hz
    explosive (pressure) source of shot `shot` (one of 16 on a 4 x 4 grid at depth L + 6; the source kind of
    layered256, for the reason given there), 16 x 16 surface receivers recording vz and p.  The medium is left to
    the device generator (extra["spec"])."""
    h, dt, f0 = 5.0, 4e-4, 25.0
    zi = n // 2
    anomaly = dict(center=(n / 2, n / 2, 0.78 * zi), radius=100.0 / h, dkdry=-0.10, kappa_factor=10.0)
    spec = dict(layers=[SANDSTONE, STIFF], interfaces=(zi,), seed=1234, corr_cells=10.0, pct=0.0,
                log_kappa_sigma=0.0, anomaly=anomaly if true_model else None)
    ax = np.linspace(cpml + 4, n - cpml - 5, nrec_side).round().astype(int)
    X, Y = np.meshgrid(ax, ax, indexing="xy")
    ijk, comp = line_receivers(X.ravel(), Y.ravel(), cpml + 2, [2, 12])
    grid = np.linspace(cpml + 10, n - cpml - 11, 4).round().astype(int)
    src = (int(grid[shot % 4]), int(grid[(shot // 4) % 4]), cpml + 6)
    return Problem(n, n, n, h, dt, radius, np.zeros((9, 1, 1, 1), np.float32), ricker(nt, dt, f0), src, ijk, comp,
                   src_kind="explosive", cpml_width=cpml, cpml_v0=p_velocity(STIFF), f0=f0,
                   name=f"inversion{n}", extra={"spec": spec, "shot": shot})


def random1024(n=1024, nt=3000, radius=4, cpml=20, nrec_side=512, seed=1234, medium=True) -> Problem:
    """The 1024^3 random medium; with medium=False the moduli are left for the device generator."""
    h, dt, f0 = 5.0, 4e-4, 20.0
    shape = (n, n, n)
    mod = random_medium(shape, seed=seed) if medium else np.zeros((9, 1, 1, 1), np.float32)
    spec = random_spec(seed=seed)
    c = n // 2
    ax = np.linspace(cpml + 2, n - cpml - 3, nrec_side).round().astype(int)
    X, Y = np.meshgrid(ax, ax, indexing="xy")
    ijk, comp = line_receivers(X.ravel(), Y.ravel(), cpml + 2, [2, 12])
    src = (c, c, min(n // 4, n - cpml - 6))
    return Problem(n, n, n, h, dt, radius, mod, ricker(nt, dt, f0), src, ijk, comp, src_kind="force_z",
                   cpml_width=cpml, cpml_v0=p_velocity(SANDSTONE) * 1.1, f0=f0, name=f"random{n}",
                   extra={"seed": seed, "spec": spec})


def borehole_moduli(nz, ny, nx) -> np.ndarray:
    """The reference's borehole medium (outputfunc.cpp:153-222) with its float/double rounding."""
    out = np.zeros((9, nz, ny, nx), np.float32)
    iy, ix = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    fluid = ((ix - nx // 2) ** 2 + (iy - ny // 2) ** 2) <= 100
    f32 = np.float32
    # formation (float volumes, double rock constants, HH from the float-rounded M)
    vp, vs, rhos, rhof, vf, por = f32(5000), f32(3300), f32(2450), f32(1000), f32(1500), 0.1
    rho = f32((1 - por) * rhos + por * rhof)
    mu = f32((1 - por) * float(rhos) * float(vs) * float(vs))
    kb = float(rhos) * (1 - por) * (float(f32(vp * vp)) - float(f32(vs * vs)) * 4.0 / 3.0)
    ks = float(rhos) * (float(f32(vp * vp)) - float(f32(vs * vs)) * 4.0 / 3.0)
    kf = float(f32(f32(rhof * vf) * vf))
    a1 = 1 - kb / ks
    M = f32(kf * ks / (por * ks + (a1 - por) * kf))
    HH = f32(a1 * a1 * float(M) + kb + float(mu) * 4.0 / 3.0)
    form = [rho, rhof, mu, M, f32(float(M) * a1), HH, f32(HH - f32(2) * mu), f32(1e-3 / (2e-12)),
            f32((1 + 2 / 8.0) * 3.0 * float(rhof) / por)]
    kff = f32(f32(f32(1000) * f32(1500)) * f32(1500))
    flu = [f32(1000), f32(1000), f32(0), kff, kff, kff, kff, f32(0), f32(1000)]
    for q in range(9):
        out[q] = np.where(fluid, flu[q], form[q])[None]
    return out


def borehole(scale: float = 1.0, nt=3500) -> Problem:
    """The reference's problem (main.cpp:20-23, 84-99), optionally shrunk by ``scale`` (cells): txx recorded
    on the whole vertical line through the source (the reference's sisx files hold every z of that line)."""
    NX, NY, NZ = (max(24, int(round(v * scale))) for v in (180, 180, 300))
    NP = max(4, int(round(30 * scale)))
    nx, ny, nz = NX + 2 * NP, NY + 2 * NP, NZ + 2 * NP
    h, dt, f0 = 0.01, 1e-6, 1e4
    sx, sy, sz = nx // 2, ny // 2, min(20 + NP, nz - NP - 2)
    ijk, comp = line_receivers(sx, sy, np.arange(0, nz), [6])
    return Problem(nx, ny, nz, h, dt, 1, borehole_moduli(nz, ny, nx), ricker_reference(nt, dt, f0), (sx, sy, sz),
                   ijk, comp, cpml_width=NP, cpml_v0=4000.0, cpml_r=1e-6, f0=f0, ref_bug_compat=True,
                   scales=(1e8, 1e8, 1.0, 1.0), name="borehole")


WORKLOADS = {"small64": small64, "layered256": layered256, "random1024": random1024, "borehole": borehole,
             "inversion256": inversion256}
