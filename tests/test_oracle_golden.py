"""CPU: the oracle against the reference's own kernels (golden fixtures) and its own consistency.

The fixtures in tests/golden were produced by the reference's Source/FD_Vbottom/FD_Tbottom kernel
bodies and create_model_all compiled for the CPU (tests/golden/make_golden.py).  The oracle's
reference-arithmetic mode must reproduce them bit for bit.
"""
import numpy as np
import pytest

from conftest import load_golden

CASES = ["ref_borehole", "ref_rock"]


@pytest.mark.parametrize("case", CASES)
def test_ref_mode_bit_exact_vs_reference_kernels(oracle, case):
    g = load_golden(case)
    nz, ny, nx = (int(v) for v in g["shape"])
    state = np.zeros((16, nz, ny, nx), np.uint16)
    aux = np.zeros((48, nz, ny, nx), np.uint16)
    seis = oracle.ref_run((nz, ny, nx), float(g["dt"]), int(g["nt"]), int(g["sn"]), g["wavelet"], state,
                          np.ascontiguousarray(g["coef"]), np.ascontiguousarray(g["prof"]), aux, g["rec_lin"],
                          g["rec_comp"])
    assert np.any(g["state"] != 0)
    for i in range(16):
        nbad = int(np.count_nonzero(state[i] != g["state"][i]))
        assert nbad == 0, f"state array {i}: {nbad} cells differ from the reference kernels"
    names = oracle.ref_aux_names()
    for i in range(48):
        nbad = int(np.count_nonzero(aux[i] != g["aux"][i]))
        assert nbad == 0, f"CPML array {names[i]}: {nbad} cells differ"
    np.testing.assert_array_equal(seis, g["seis"])


def test_ref_inputs_reproduce_fixture_inputs(oracle):
    """The oracle's restatement of main.cpp's coefficient/CPML build gives the fixture's FP16 inputs."""
    g = load_golden("ref_borehole")
    coef, prof = oracle.ref_inputs(g["medium"], float(g["h"]), float(g["dt"]), int(g["np_cells"]))
    np.testing.assert_array_equal(coef, g["coef"])
    np.testing.assert_array_equal(prof, g["prof"])


def test_borehole_medium_matches_reference(oracle):
    g = load_golden("ref_borehole")
    nz, ny, nx = (int(v) for v in g["shape"])
    mine = oracle.medium_borehole(nz, ny, nx)
    np.testing.assert_array_equal(mine, g["medium"])


def test_product_borehole_medium_matches_oracle(oracle):
    from behf import problems
    a = problems.borehole_moduli(12, 30, 32)
    np.testing.assert_array_equal(a, oracle.medium_borehole(12, 30, 32))


def test_rock_moduli_match(oracle):
    from behf import problems
    for rock in (problems.SANDSTONE, problems.STIFF):
        np.testing.assert_allclose(problems.rock_moduli(**rock), oracle.rock_moduli(**rock), rtol=1e-15)


def test_behf_fp64_r1_tracks_reference_scheme(oracle):
    """The BEHF scheme at radius 1 with the reference's bug-compatible vz update and scales is the
    reference's equations: its FP64 run stays within FP16 rounding of the reference kernels' run."""
    from behf import problems
    g = load_golden("ref_rock")
    nz, ny, nx = (int(v) for v in g["shape"])
    sx, sy, sz = (int(v) for v in g["src"])
    rec_lin = g["rec_lin"].astype(np.int64)
    ijk = np.stack([rec_lin % nx, (rec_lin // nx) % ny, rec_lin // (nx * ny)], 1).astype(np.int32)
    prob = problems.Problem(nx, ny, nz, float(g["h"]), float(g["dt"]), 1, g["medium"], g["wavelet"], (sx, sy, sz),
                            ijk, g["rec_comp"], cpml_width=int(g["np_cells"]), cpml_v0=4000.0, cpml_r=1e-6,
                            ref_bug_compat=True, scales=(1e8, 1e8, 1.0, 1.0))
    seis, _ = oracle.run(prob, "f64")
    ref = g["seis"].astype(np.float64)
    scale = np.array([1e8 if c < 6 else 1.0 for c in g["rec_comp"]])[:, None]
    for comp in np.unique(g["rec_comp"]):
        sel = g["rec_comp"] == comp
        err = oracle.rel_l2(seis[sel] * scale[sel], ref[sel])
        assert err < 5e-2, f"field {comp}: rel-L2 {err:.3e} between FP64 BEHF and the FP16 reference"


def test_stencil_order(oracle):
    """Radius R gives order 2R: a plane wave's phase error falls with R (sanity of the weights)."""
    from behf import problems
    errs = []
    for R in (1, 2, 4):
        p = problems.small64(n=36, nt=120, radius=R, cpml=8)
        s, _ = oracle.run(p, "f64")
        errs.append(s)
    # higher orders agree with each other much better than with second order
    d12 = oracle.rel_l2(errs[0], errs[2])
    d24 = oracle.rel_l2(errs[1], errs[2])
    assert d24 < 0.5 * d12
