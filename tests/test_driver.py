"""Command-line driver and output formats, on the CPU: the text layout of the reference's wfile/wfile3d,
the binary layout, and the driver's problem set-up (--setup-only touches no GPU) against the Python
problem descriptions that the GPU parity tests run."""
from __future__ import annotations

import json
import subprocess

import numpy as np
import pytest

from behf import io as bio
from behf import problems


@pytest.fixture(scope="module")
def driver():
    from behf import build
    return str(build.build_driver())


def test_wfile_text_layout(tmp_path):
    p = tmp_path / "a.dat"
    bio.write_wfile(p, [[1.0, -2.5, 3e-7], [0.0, 1e10, -4.25]])
    # outputfunc.cpp:35-50: "%e " per value, "\n" after the last column, "\n" after each row
    assert p.read_text() == ("1.000000e+00 -2.500000e+00 3.000000e-07 \n\n"
                             "0.000000e+00 1.000000e+10 -4.250000e+00 \n\n")
    np.testing.assert_array_equal(bio.read_wfile(p), np.float32([[1.0, -2.5, 3e-7], [0.0, 1e10, -4.25]]))


def test_wfile3d_is_the_y_mid_slice(tmp_path):
    v = np.arange(3 * 5 * 4, dtype=np.float32).reshape(3, 5, 4)
    p = tmp_path / "s.dat"
    bio.write_wfile3d(p, v)
    np.testing.assert_array_equal(bio.read_wfile(p), v[:, 2, :])


def test_binary_roundtrip_and_checks(tmp_path):
    a = np.random.default_rng(0).standard_normal((7, 11)).astype(np.float32)
    bio.write_binary(tmp_path / "a.bin", a)
    np.testing.assert_array_equal(bio.read(tmp_path / "a.bin"), a)
    i = np.arange(12, dtype=np.int64).reshape(3, 4)
    bio.write_binary(tmp_path / "i.bin", i)
    r = bio.read_binary(tmp_path / "i.bin")
    assert r.dtype == np.int32
    np.testing.assert_array_equal(r, i)
    raw = (tmp_path / "a.bin").read_bytes()
    (tmp_path / "bad.bin").write_bytes(b"NOTBEHF!" + raw[8:])
    with pytest.raises(ValueError):
        bio.read_binary(tmp_path / "bad.bin")
    (tmp_path / "short.bin").write_bytes(raw[:-4])
    with pytest.raises(ValueError):
        bio.read_binary(tmp_path / "short.bin")


def test_driver_usage_errors(driver):
    r = subprocess.run([driver, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "usage" in r.stdout
    for bad in (["--precision", "f8"], ["--bogus", "1"], ["--snap-field", "nope"], ["--format", "xml"], ["--nt"],
                ["--variant", "fast"]):
        r = subprocess.run([driver, *bad], capture_output=True, text=True)
        assert r.returncode == 1, bad
    r = subprocess.run([driver, "--preset", "nope", "--setup-only", "--out", "/tmp"], capture_output=True, text=True)
    assert r.returncode == 1


def _setup(driver, tmp_path, *args):
    r = subprocess.run([driver, *args, "--setup-only", "--out", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("scale", [0.2, 0.5])
def test_driver_borehole_setup_matches_problem(driver, tmp_path, scale):
    nt = 400
    meta = _setup(driver, tmp_path, "--preset", "borehole", "--scale", str(scale), "--nt", str(nt))
    prob = problems.borehole(scale, nt)
    assert meta["grid"] == [prob.nx, prob.ny, prob.nz]
    assert meta["radius"] == 1 and meta["cpml_width"] == prob.cpml_width and meta["ref_bug_compat"]
    assert meta["src"] == list(prob.src) and meta["scales"] == list(prob.scales)
    assert meta["h"] == prob.h and meta["dt"] == prob.dt and meta["cpml_v0"] == prob.cpml_v0
    np.testing.assert_array_equal(bio.read(tmp_path / "wavelet.bin"), prob.wavelet)
    np.testing.assert_array_equal(bio.read(tmp_path / "moduli.bin"), prob.mod)
    rec = bio.read(tmp_path / "receivers.bin")
    np.testing.assert_array_equal(rec[:, :3], prob.rec_ijk)
    np.testing.assert_array_equal(rec[:, 3], prob.rec_comp)


def test_driver_borehole_medium_matches_oracle(driver, tmp_path, oracle):
    _setup(driver, tmp_path, "--preset", "borehole", "--scale", "0.2", "--nt", "10")
    mod = bio.read(tmp_path / "moduli.bin")
    np.testing.assert_array_equal(mod, oracle.medium_borehole(*mod.shape[1:]))


def test_driver_cube_presets(driver, tmp_path):
    meta = _setup(driver, tmp_path, "--preset", "layered256", "--scale", "0.25", "--nt", "50")
    assert meta["grid"] == [64, 64, 64] and meta["radius"] == 4 and not meta["host_medium"]
    rec = bio.read(tmp_path / "receivers.bin")
    assert rec.shape == (2 * 16 * 16, 4) and set(rec[:, 3]) == {2, 12}
    assert (rec[:, :3] >= 0).all() and (rec[:, :3] < 64).all()
    w = bio.read(tmp_path / "wavelet.bin")
    np.testing.assert_allclose(w, problems.ricker(50, 4e-4, 25.0), rtol=0, atol=1e-6)
    meta = _setup(driver, tmp_path, "--preset", "random1024", "--scale", "0.125", "--nt", "20")
    assert meta["grid"] == [128, 128, 128] and meta["src_kind"] == 2
