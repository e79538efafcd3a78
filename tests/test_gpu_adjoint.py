"""Adjoint-state gradient on the GPU (behf_gradient / behf_misfit_gradient through the C ABI), against the
FP64 CPU discrete adjoint of the oracle (itself pinned by the dot-product identity and finite differences):
  * FP64: wavelet and moduli gradients within 1e-9 relative L2 of the oracle, every source kind, radius 1/2/4,
    with and without CPML; dot-product identity within 1e-10; checkpoint spacing, two checkpoint levels and the
    snapshot cache, the overlap of the recompute with the adjoint steps, the L2 prefetch and the memory updates in
    the gradient kernels change nothing;
  * FP32 storage + FP32 adjoint: within 1e-4 of the oracle; FP16 storage (FP32 adjoint): within 5e-2; BF16
    storage within 0.35;
  * finite differences of the GPU's own FP64 misfit agree with its gradient within 1e-3."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

import behf
from behf import problems as P

pytestmark = pytest.mark.gpu


def small(n=22, nt=70, R=2, L=4, kind="explosive"):
    p = P.small64(n=n, nt=nt, radius=R, cpml=L)
    mod = P.layered((n, n, n), [P.SANDSTONE, P.STIFF], [n // 2 + 2])
    rng = np.random.default_rng(1)
    ijk = rng.integers(R + 1, n - R - 1, size=(12, 3)).astype(np.int32)
    comp = rng.integers(0, 13, size=12).astype(np.int32)
    return dataclasses.replace(p, mod=mod, src_kind=kind, scales=(1, 1, 1, 1), rec_ijk=ijk, rec_comp=comp)


def rel(a, b):
    d = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / d if d > 0 else np.linalg.norm(a.ravel())


def gpu_gradient(p, adj, precision, checkpoint=0, kernel="auto", snapshot_cache=-1, checkpoint_outer=0, overlap=1):
    s = behf.solver_for(p, precision=precision, kernel=kernel, gradient=True, checkpoint=checkpoint,
                        snapshot_cache=snapshot_cache, checkpoint_outer=checkpoint_outer, overlap=overlap)
    gw, gm = s.gradient(p.nt, adj)
    seis = s.seismograms()
    s.close()
    return seis, gw, gm


CASES = [("explosive", 2, 4), ("pressure", 1, 0), ("force_z", 4, 5)]


@pytest.mark.parametrize("kind,R,L", CASES)
def test_gradient_f64_matches_oracle(behf_lib, oracle, kind, R, L):
    p = small(R=R, L=L, kind=kind)
    adj = np.random.default_rng(4).standard_normal((len(p.rec_comp), p.nt))
    ref = oracle.adjoint(p, adj, stride=8)
    seis, gw, gm = gpu_gradient(p, adj, "f64")
    assert rel(seis, ref["seis"]) < 1e-10
    assert rel(gw, ref["grad_wavelet"]) < 1e-9
    for q in range(9):
        assert rel(gm[q], ref["grad_mod"][q]) < 1e-8, q
    assert not gm[:, : max(R, L) + 1].any()  # outside the inverted region


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32", 1e-4)])
def test_gradient_dot_product(behf_lib, precision, tol):
    p = small(R=4, L=5, kind="force_z")
    rng = np.random.default_rng(5)
    w = rng.standard_normal(p.nt).astype(np.float32)
    p = dataclasses.replace(p, wavelet=w)
    s = behf.solver_for(p, precision=precision, gradient=True)
    s.run(p.nt)
    d = s.seismograms()
    r = rng.standard_normal(d.shape)
    lt, _ = s.gradient(p.nt, r, moduli=False)
    s.close()
    lhs, rhs = float((d * r).sum()), float((w.astype(np.float64) * lt).sum())
    assert abs(lhs - rhs) <= tol * abs(lhs)


def test_gradient_checkpoint_spacing(behf_lib):
    p = small(R=2, L=4)
    adj = np.random.default_rng(6).standard_normal((len(p.rec_comp), p.nt))
    _, gw1, gm1 = gpu_gradient(p, adj, "f64", checkpoint=1)
    _, gw2, gm2 = gpu_gradient(p, adj, "f64", checkpoint=13)
    _, gw3, gm3 = gpu_gradient(p, adj, "f64", checkpoint=p.nt)
    for a, b in ((gw1, gw2), (gw1, gw3), (gm1, gm2), (gm1, gm3)):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())


@pytest.mark.parametrize("switch", ["BEHF_ADJ_PREFETCH", "BEHF_ADJ_VMERGE", "BEHF_RC_OOP"])
@pytest.mark.parametrize("precision", ["f32", "f16"])
def test_gradient_kernel_switches_change_nothing(behf_lib, precision, switch, monkeypatch):
    # the adjoint kernels' L2 prefetch of the next plane only moves data into L2, the CPML memory updates done
    # by the gradient kernels for their slab cells are k_vmem's arithmetic, and the out-of-place recompute writes
    # the snapshot slots the copies would fill: all on by default, =0 turns one off; the same gradient, bit for bit
    p = small(R=4, L=5, kind="force_z")
    adj = np.random.default_rng(11).standard_normal((len(p.rec_comp), p.nt))
    monkeypatch.setenv(switch, "0")
    ref = gpu_gradient(p, adj, precision, checkpoint=13, snapshot_cache=0)  # every segment recomputed
    monkeypatch.setenv(switch, "1")
    out = gpu_gradient(p, adj, precision, checkpoint=13, snapshot_cache=0)
    for a, b in zip(out, ref):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision", ["f64", "f32", "f16"])
def test_gradient_snapshot_cache(behf_lib, precision):
    # every segment recomputed (0), the last two kept from the forward pass (50 MiB of 1.6 MB slots x 13 per
    # segment at f64), all kept (-1): the same gradient, bit for bit; and the recomputes overlapped with the
    # adjoint steps on a second stream (the default) or run one after the other
    p = small(R=2, L=4)
    adj = np.random.default_rng(7).standard_normal((len(p.rec_comp), p.nt))
    ref = gpu_gradient(p, adj, precision, checkpoint=13, snapshot_cache=0, overlap=0)
    for cache in (0, 50, -1):
        for overlap in (0, 1):
            if (cache, overlap) == (0, 0):
                continue
            out = gpu_gradient(p, adj, precision, checkpoint=13, snapshot_cache=cache, overlap=overlap)
            for a, b in zip(out, ref):
                np.testing.assert_array_equal(a, b)
    # two checkpoint levels (outer segments of 39 = 3 x 13 steps, each run again for its inner checkpoints)
    out = gpu_gradient(p, adj, precision, checkpoint=13, checkpoint_outer=30)
    for a, b in zip(out, ref):
        np.testing.assert_array_equal(a, b)


# measured (this problem): FP16 moduli and parameters within 2.6e-2, BF16 within 0.27 (three fewer stored
# significand bits); the wavelet gradient (3.5e-3) does not depend on the stored forward fields
@pytest.mark.parametrize("precision,tol", [("f32", 1e-4), ("f16", 5e-2), ("bf16", 0.35)])
def test_gradient_reduced_precision(behf_lib, oracle, precision, tol):
    p = small(R=4, L=5, kind="explosive")
    adj = np.random.default_rng(7).standard_normal((len(p.rec_comp), p.nt))
    ref = oracle.adjoint(p, adj)
    _, gw, gm = gpu_gradient(p, adj, precision)
    assert rel(gw, ref["grad_wavelet"]) < tol
    for q in range(9):
        assert rel(gm[q], ref["grad_mod"][q]) < tol, q
    gp, gp_ref = behf.physical_gradient(p.mod, gm), behf.physical_gradient(p.mod, ref["grad_mod"])
    for q in range(7):
        assert rel(gp[q], gp_ref[q]) < tol, behf.PHYSICAL[q]


def test_misfit_gradient_and_finite_differences(behf_lib):
    p = small(n=24, nt=80, R=2, L=4, kind="explosive")
    n = p.nx
    zz, yy, xx = np.meshgrid(*[np.arange(n)] * 3, indexing="ij")
    blob = np.exp(-((xx - n / 2) ** 2 + (yy - n / 2 - 1) ** 2 + (zz - n / 2 + 1) ** 2) / 6.0)
    mtrue = p.mod.copy()
    mtrue[5] *= (1 + 0.05 * blob).astype(np.float32)

    def forward(mod):
        s = behf.solver_for(dataclasses.replace(p, mod=mod), precision="f64")
        s.run(p.nt)
        d = s.seismograms()
        s.close()
        return d

    dobs = forward(mtrue)
    s = behf.solver_for(p, precision="f64", gradient=True)
    J, gw, gm = s.misfit_gradient(p.nt, dobs)
    s.close()
    d0 = forward(p.mod)
    assert abs(J - 0.5 * ((d0 - dobs) ** 2).sum()) <= 1e-12 * J
    for q in (0, 5):
        base = p.mod[q].astype(np.float64)
        mp, mm = p.mod.copy(), p.mod.copy()
        mp[q] = (base * (1 + 1e-3 * blob)).astype(np.float32)
        mm[q] = (base * (1 - 1e-3 * blob)).astype(np.float32)
        fd = 0.5 * ((forward(mp) - dobs) ** 2).sum() - 0.5 * ((forward(mm) - dobs) ** 2).sum()
        pred = float((gm[q] * (mp[q].astype(np.float64) - mm[q].astype(np.float64))).sum())
        assert abs(fd - pred) <= 1e-3 * abs(fd), (q, fd, pred)


def test_gradient_errors(behf_lib):
    p = small()
    s = behf.solver_for(p, precision="f32")
    with pytest.raises(behf.BehfError) as e:
        s.gradient(p.nt, np.zeros((len(p.rec_comp), p.nt)))
    assert e.value.code == -4  # BEHF_ERR_STATE: gradient support not enabled before the medium
    with pytest.raises(behf.BehfError):
        s.enable_gradient()  # too late: the medium is set
    s.close()
    s = behf.solver_for(p, precision="f32", gradient=True, capacity=p.nt - 1)
    with pytest.raises(behf.BehfError):
        s.gradient(p.nt, np.zeros((len(p.rec_comp), p.nt)))
    s.close()


def test_torch_autograd_wrapper(behf_lib):
    torch = pytest.importorskip("torch")
    from behf import torch_ops
    p = small(R=2, L=4, kind="explosive")
    rng = np.random.default_rng(8)
    dobs = rng.standard_normal((len(p.rec_comp), p.nt)) * 1e-3
    sim = torch_ops.Simulation(p, precision="f64")
    mod = torch.tensor(p.mod, device="cuda", requires_grad=True)
    w = torch.tensor(p.wavelet, requires_grad=True)
    seis = sim(mod, w)
    loss = 0.5 * ((seis - torch.from_numpy(dobs)) ** 2).sum()
    loss.backward()
    sim.close()
    s = behf.solver_for(p, precision="f64", gradient=True)
    J, gw, gm = s.misfit_gradient(p.nt, dobs)
    s.close()
    assert abs(loss.item() - J) <= 1e-10 * J
    assert rel(mod.grad.double().cpu().numpy(), gm.astype(np.float32).astype(np.float64)) < 1e-6
    assert rel(w.grad.double().numpy(), gw.astype(np.float32).astype(np.float64)) < 1e-6


def _inversion_case(n=48, nt=300, true_model=False, cpml=8):
    """The gradient workload (two-layer medium, 100 m anomaly of -10 % K_dry and x10 kappa in the true model,
    pressure source, surface receivers of vz and p) on n^3 cells of 5 m, with host moduli."""
    p = P.inversion256(n=n, nt=nt, true_model=true_model, cpml=cpml, nrec_side=8)
    sp = p.extra["spec"]
    mod = P.spec_medium((n, n, n), sp["layers"], sp["interfaces"], sp["seed"], sp["corr_cells"], sp["pct"],
                        sp["log_kappa_sigma"], sp["anomaly"])
    return dataclasses.replace(p, mod=mod)


def test_gradient_48_matches_cpu_fp64_adjoint(behf_lib, oracle):
    """The 48^3 sub-case of the gradient workload: the GPU gradient (FP64 storage) against the FP64 CPU discrete
    adjoint of the oracle, in the moduli and in the physical parameters."""
    p = _inversion_case()
    dobs = oracle.run(_inversion_case(true_model=True), "f64")[0]
    s = behf.solver_for(p, precision="f64", gradient=True)
    J, gw, gm = s.misfit_gradient(p.nt, dobs)
    seis = s.seismograms()
    s.close()
    assert J > 0
    ref = oracle.adjoint(p, seis - dobs)
    assert rel(gw, ref["grad_wavelet"]) < 1e-9
    for q in range(9):
        assert rel(gm[q], ref["grad_mod"][q]) < 1e-8, q
    gp, gp_ref = behf.physical_gradient(p.mod, gm), behf.physical_gradient(p.mod, ref["grad_mod"])
    for q in range(7):
        assert np.abs(gp_ref[q]).max() > 0, behf.PHYSICAL[q]
        assert rel(gp[q], gp_ref[q]) < 1e-8, behf.PHYSICAL[q]


@pytest.mark.parametrize("seed", range(8))
def test_physical_gradient_central_differences(behf_lib, seed):
    """Central differences of the FP64 misfit along a random seeded direction that perturbs all seven physical
    parameters of every cell of the inverted region at once (relative steps +-1e-3)."""
    p = _inversion_case(n=26, nt=120, cpml=4)
    n = p.nx
    dobs = _forward_f64(_inversion_case(n=26, nt=120, true_model=True, cpml=4))
    s = behf.solver_for(p, precision="f64", gradient=True)
    J, _, gm = s.misfit_gradient(p.nt, dobs)
    s.close()
    gp = behf.physical_gradient(p.mod, gm)
    phys, ratio = P.physical_from_moduli(p.mod)
    rng = np.random.default_rng(100 + seed)
    d = rng.standard_normal(phys.shape)
    m = p.cpml_width + p.radius + 2  # the inverted region (cells whose coefficient cells lie outside the slabs)
    mask = np.zeros((n, n, n), bool)
    mask[m:n - m, m:n - m, m:n - m] = True
    d *= mask
    eps = 1e-3
    php, phm = phys * (1 + eps * d), phys * (1 - eps * d)
    jp = 0.5 * ((_forward_f64(dataclasses.replace(p, mod=P.moduli_from_physical(php, ratio))) - dobs) ** 2).sum()
    jm = 0.5 * ((_forward_f64(dataclasses.replace(p, mod=P.moduli_from_physical(phm, ratio))) - dobs) ** 2).sum()
    fd = jp - jm
    pred = float((gp * (php - phm)).sum())
    assert abs(fd - pred) <= 1e-3 * abs(fd), (fd, pred)


def _forward_f64(p):
    s = behf.solver_for(p, precision="f64")
    s.run(p.nt)
    d = s.seismograms()
    s.close()
    return d


def test_gradient_compensated_accumulation(behf_lib, oracle):
    """FP32 adjoint over 400 steps: the Neumaier-folded accumulators (the default) are at least as close to the
    FP64-folded ones as plain FP32 accumulation over all steps; the two folded modes stay within 1e-4 of the FP64
    oracle, plain accumulation within 1e-3 (measured 2.5e-4 on the m gradient)."""
    p = small(n=22, nt=400, R=2, L=4, kind="explosive")
    adj = np.random.default_rng(9).standard_normal((len(p.rec_comp), p.nt))
    ref = oracle.adjoint(p, adj)
    out = {}
    for mode in (0, 1, 2):
        s = behf.solver_for(p, precision="f32", gradient=True, checkpoint=20)
        s.set_option(behf.OPT_GRAD_COMPENSATION, mode)
        _, gm = s.gradient(p.nt, adj)
        s.close()
        out[mode] = gm
    for q in range(9):
        e_plain, e_comp = rel(out[0][q], out[2][q]), rel(out[1][q], out[2][q])
        assert e_comp <= e_plain + 1e-9, (q, e_plain, e_comp)
        for mode, tol in ((0, 1e-3), (1, 1e-4), (2, 1e-4)):
            assert rel(out[mode][q], ref["grad_mod"][q]) < tol, (q, mode)
