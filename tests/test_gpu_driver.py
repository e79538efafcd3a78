"""The command-line driver on the GPU: the reference's borehole problem (shrunk) run by behf_run must give
the same seismograms and snapshots as the same problem run through the Python API (same library, same
inputs: identical up to the 7 significant digits of the text layout), in both output layouts."""
from __future__ import annotations

import json
import subprocess

import numpy as np
import pytest

import behf
from behf import io as bio
from behf import problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(behf_lib):
    from behf import build
    return str(build.build_driver())


def _run(driver, out, *args):
    r = subprocess.run([driver, *args, "--out", str(out), "--quiet"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_driver_borehole_matches_api(driver, tmp_path):
    nt, snap = 300, 149
    meta = _run(driver, tmp_path, "--preset", "borehole", "--scale", "0.2", "--nt", str(nt), "--snap", str(snap),
                "--format", "both")
    assert meta["health_ok"] and meta["steps"] == nt
    prob = problems.borehole(0.2, nt)
    s = behf.solver_for(prob, precision="f16", scales=prob.scales)
    s.run(snap + 1)
    snap_api = s.get_field("sxx")[:, prob.ny // 2, :]
    s.run(nt - snap - 1)
    seis = s.seismograms().astype(np.float32)
    s.close()
    for ext in (".bin", ".dat"):
        got = bio.read(tmp_path / f"sis_txx{ext}")
        assert got.shape == (prob.nz, nt)
        got_snap = bio.read(tmp_path / f"txxpro_{snap}{ext}")
        assert got_snap.shape == (prob.nz, prob.nx)
        if ext == ".bin":
            np.testing.assert_array_equal(got, seis)
            np.testing.assert_array_equal(got_snap, snap_api)
        else:  # "%e": 7 significant digits
            np.testing.assert_allclose(got, seis, rtol=6e-7, atol=0)
            np.testing.assert_allclose(got_snap, snap_api, rtol=6e-7, atol=0)
    assert np.abs(seis).max() > 0 and np.isfinite(seis).all()


def test_driver_cube_preset_runs(driver, tmp_path):
    meta = _run(driver, tmp_path, "--preset", "layered256", "--scale", "0.25", "--nt", "120", "--snap", "60",
                "--snap-field", "p", "--format", "binary", "--precision", "f32")
    assert meta["health_ok"] and meta["grid"] == [64, 64, 64] and meta["precision"] == 1
    vz, p = bio.read(tmp_path / "sis_vuz.bin"), bio.read(tmp_path / "sis_ss.bin")
    assert vz.shape == (256, 120) and p.shape == (256, 120)
    assert np.isfinite(vz).all() and np.abs(p).max() > 0
    assert bio.read(tmp_path / "sspro_60.bin").shape == (64, 64)


def test_driver_variant_option(driver, tmp_path):
    """--variant selects the tiled-kernel variant; the tensor-memory variants with and without the x-slab staging
    give the same bits."""
    out = {}
    for v in ("tmem", "tmem_xs"):
        d = tmp_path / v
        meta = _run(driver, d, "--preset", "layered256", "--scale", "0.5", "--nt", "60", "--snap", "30",
                    "--format", "binary", "--precision", "f16", "--variant", v)
        assert meta["health_ok"]
        out[v] = bio.read(d / "sis_vuz.bin")
    np.testing.assert_array_equal(out["tmem"], out["tmem_xs"])
