"""behf_physical_gradient on the CPU (host arithmetic only): the chain rule from the moduli gradients to Biot's
physical parameters (lambda, mu, rho, rho_f, M, alpha, kappa), checked against central differences of a linear
functional of the moduli, J(p) = sum g_mod . moduli(p), along random directions, and the round trip of the
parameter maps."""
from __future__ import annotations

import numpy as np
import pytest

import behf
from behf import problems as P


def _medium(shape=(6, 7, 8)):
    """Two layers with correlated perturbations of K_dry, mu, phi and log-normal kappa (consistent moduli)."""
    return P.spec_medium(shape, [P.SANDSTONE, P.STIFF], (shape[0] // 2,), seed=3, corr_cells=2.0, pct=0.05,
                         log_kappa_sigma=0.5)


def test_parameter_maps_round_trip():
    mod = _medium()
    phys, ratio = P.physical_from_moduli(mod)
    back = P.moduli_from_physical(phys, ratio)
    np.testing.assert_allclose(back, mod, rtol=2e-6)


@pytest.mark.parametrize("seed", range(4))
def test_chain_rule_matches_central_differences(seed):
    mod = _medium()
    rng = np.random.default_rng(seed)
    gm = rng.standard_normal(mod.shape)
    gm[:, 0, 0, 0] = 0.0  # a cell outside the inverted region
    gp = behf.physical_gradient(mod, gm)
    phys, ratio = P.physical_from_moduli(mod)

    def J(ph):  # linear in the moduli, which are smooth functions of the parameters (FP64 throughout)
        lam, mu, rho, rhof, M, alpha, kappa = ph
        h2u = lam + alpha * alpha * M
        mods = np.stack([rho, rhof, mu, M, alpha * M, h2u + 2 * mu, h2u, 1e-3 / kappa, ratio * rhof])
        return float((gm * mods).sum())

    d = rng.standard_normal(phys.shape) * np.abs(phys)  # relative perturbation of every parameter in every cell
    eps = 1e-6
    fd = (J(phys + eps * d) - J(phys - eps * d)) / (2 * eps)
    pred = float((gp * d).sum())
    assert abs(fd - pred) <= 1e-6 * max(abs(fd), np.abs(gp * d).sum()), (fd, pred)
    assert not gp[:, 0, 0, 0].any()


def test_fluid_cells():
    mod = P.borehole_moduli(2, 24, 24)  # fluid-filled borehole: mu = 0, b = 0, C = M = K_f
    gm = np.ones(mod.shape)
    gp = behf.physical_gradient(mod, gm)
    fluid = mod[7] == 0
    assert fluid.any()
    assert not gp[6][fluid].any()  # no permeability gradient in pure fluid
    # alpha = 1 there: g_alpha = M g_C + 2 M (g_H + g_lambda_u)
    M = mod[3].astype(np.float64)
    np.testing.assert_allclose(gp[5][fluid], (M + 4 * M)[fluid], rtol=1e-12)


def test_bad_arguments():
    mod = _medium()
    with pytest.raises(behf.BehfError):
        behf.physical_gradient(mod, np.zeros(mod.shape), eta=0.0)
    with pytest.raises(ValueError):
        behf.physical_gradient(mod, np.zeros((9, 1, 1, 1)))
