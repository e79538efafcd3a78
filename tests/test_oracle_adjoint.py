"""The FP64 CPU discrete adjoint (oracle/behf_adjoint.cpp), on the CPU: it is the checker of the CUDA
adjoint, so it is pinned first by the two properties an exact discrete adjoint must have:
  * dot-product identity <L w, r> = <w, L^T r> for the linear map L from source wavelet to seismograms
    (every source kind, radius 1/2/4, with and without CPML): relative error <= 1e-12;
  * central finite differences of the L2 misfit J = 1/2 |d(m) - d_obs|^2 along a smooth perturbation of
    each cell-centred modulus agree with <grad J, dm>: relative error <= 1e-3.
Its forward must equal orc_run in FP64 bit for bit, and the result may not depend on the checkpoint stride."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from behf import problems as P

MODULI = ["rho", "rhof", "mu", "M", "C", "HH", "H2U", "C1", "C2"]


def small(n=22, nt=70, R=2, L=4, kind="explosive"):
    p = P.small64(n=n, nt=nt, radius=R, cpml=L)
    mod = P.layered((n, n, n), [P.SANDSTONE, P.STIFF], [n // 2 + 2])
    rng = np.random.default_rng(1)
    ijk = rng.integers(R + 1, n - R - 1, size=(12, 3)).astype(np.int32)
    comp = rng.integers(0, 13, size=12).astype(np.int32)
    return dataclasses.replace(p, mod=mod, src_kind=kind, scales=(1, 1, 1, 1), rec_ijk=ijk, rec_comp=comp)


@pytest.mark.parametrize("kind,R,L", [("explosive", 2, 4), ("pressure", 1, 0), ("force_z", 4, 5)])
def test_adjoint_dot_product(oracle, kind, R, L):
    p = small(R=R, L=L, kind=kind)
    rng = np.random.default_rng(2)
    w = rng.standard_normal(p.nt).astype(np.float32)
    pw = dataclasses.replace(p, wavelet=w)
    fwd, _ = oracle.run(pw, "f64")
    out = oracle.adjoint(pw, None, stride=6)
    np.testing.assert_array_equal(out["seis"], fwd)
    r = rng.standard_normal(fwd.shape)
    lt = oracle.adjoint(pw, r, stride=5)["grad_wavelet"]
    lhs, rhs = float((fwd * r).sum()), float((w.astype(np.float64) * lt).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_adjoint_stride_invariance(oracle):
    p = small(R=2, L=4)
    r = np.random.default_rng(3).standard_normal((len(p.rec_comp), p.nt))
    a = oracle.adjoint(p, r, stride=1, want_coef=True)
    b = oracle.adjoint(p, r, stride=13, want_coef=True)
    np.testing.assert_array_equal(a["grad_wavelet"], b["grad_wavelet"])
    np.testing.assert_array_equal(a["grad_mod"], b["grad_mod"])
    np.testing.assert_array_equal(a["grad_coef"], b["grad_coef"])


@pytest.mark.parametrize("kind,R,L", [("explosive", 2, 4), ("force_z", 4, 5)])
def test_adjoint_gradient_vs_finite_differences(oracle, kind, R, L):
    p = small(n=24, nt=80, R=R, L=L, kind=kind)
    n = p.nx
    zz, yy, xx = np.meshgrid(*[np.arange(n)] * 3, indexing="ij")
    blob = np.exp(-((xx - n / 2) ** 2 + (yy - n / 2 - 1) ** 2 + (zz - n / 2 + 1) ** 2) / 6.0)
    mtrue = p.mod.copy()
    mtrue[5] *= (1 + 0.05 * blob).astype(np.float32)
    mtrue[0] *= (1 - 0.03 * blob).astype(np.float32)
    dobs, _ = oracle.run(dataclasses.replace(p, mod=mtrue), "f64")

    def J(mod):
        d, _ = oracle.run(dataclasses.replace(p, mod=mod), "f64")
        return 0.5 * float(((d - dobs) ** 2).sum()), d

    _, d0 = J(p.mod)
    g = oracle.adjoint(p, d0 - dobs, stride=9)["grad_mod"]
    # zero outside the inverted region: cells next to or inside the CPML slabs and the ghost ring
    lo = max(L, R) + 1
    assert not g[:, :lo].any() and not g[:, :, :lo].any() and not g[:, :, :, :lo].any()
    for q in (0, 2, 5, 6, 7):  # rho, mu, HH, H2U, C1
        base = p.mod[q].astype(np.float64)
        mp, mm = p.mod.copy(), p.mod.copy()
        mp[q] = (base * (1 + 1e-3 * blob)).astype(np.float32)
        mm[q] = (base * (1 - 1e-3 * blob)).astype(np.float32)
        fd = J(mp)[0] - J(mm)[0]
        pred = float((g[q] * (mp[q].astype(np.float64) - mm[q].astype(np.float64))).sum())
        assert abs(fd - pred) <= 1e-3 * abs(fd), (MODULI[q], fd, pred)


def test_adjoint_state_storage_emulation(oracle):
    """The FP16 adjoint-state emulation (lf_scale): no scale leaves the FP64 result unchanged; per-field scales
    that put each adjoint field's peak just below 2^14 keep the gradients of this short case within 1e-2 without
    overflow; a scale far too large overflows binary16 and is counted."""
    p = small(R=2, L=4)
    r = np.random.default_rng(3).standard_normal((len(p.rec_comp), p.nt))
    ref = oracle.adjoint(p, r)
    again = oracle.adjoint(p, r, lf_scale=None)
    np.testing.assert_array_equal(ref["grad_mod"], again["grad_mod"])
    mx = ref["lf_max"]
    assert mx.shape == (13,) and (mx > 0).all() and ref["lf_saturated"] == 0
    scale = 2.0 ** np.floor(np.log2(2.0 ** 14 / mx))
    emu = oracle.adjoint(p, r, lf_scale=scale)
    assert emu["lf_saturated"] == 0
    for q in range(9):
        d = np.linalg.norm(ref["grad_mod"][q])
        assert np.linalg.norm(emu["grad_mod"][q] - ref["grad_mod"][q]) <= 1e-2 * d, MODULI[q]
    assert not np.array_equal(emu["grad_mod"], ref["grad_mod"])  # the rounding did happen
    over = oracle.adjoint(p, r, lf_scale=scale * 2.0 ** 8)
    assert over["lf_saturated"] > 0
