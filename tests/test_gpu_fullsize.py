"""The benchmark workload at its full size on the GPU (1024^3 cells, 96 GB in FP16), checked through
size-independent properties: FP16 storage stays within the metric's 2e-2 seismogram bar of FP32 storage
over the main pulse, the health check passes, the tiled kernels run, and splitting the run changes no bit."""
from __future__ import annotations

import numpy as np
import pytest

import behf
from behf import problems

pytestmark = pytest.mark.gpu


def _run(prob, precision, split=None):
    s = behf.solver_for(prob, precision=precision)
    assert s.info()["kernel"] == "tiled"
    if split:
        s.run(split)
        s.run(prob.nt - split)
    else:
        s.run(prob.nt)
    ok, _ = s.health()
    seis = s.seismograms()
    s.close()
    return seis, ok


def test_random1024_fp16_vs_fp32_and_split(behf_lib):
    prob = problems.random1024(n=1024, nt=400, medium=False, nrec_side=2)
    # receivers 40 cells (200 m) above the source, so the main pulse reaches them within the 400 steps
    sx, sy, sz = prob.src
    xs = np.linspace(100, 924, 128).round().astype(int)
    prob.rec_ijk, prob.rec_comp = problems.line_receivers(xs, sy, sz - 40, [2, 12])
    a, ok16 = _run(prob, "f16")
    b, ok32 = _run(prob, "f32")
    assert ok16 and ok32
    for comp in np.unique(prob.rec_comp):
        sel = prob.rec_comp == comp
        err = np.linalg.norm(a[sel] - b[sel]) / np.linalg.norm(b[sel])
        assert err < 2e-2, (int(comp), err)
    c, _ = _run(prob, "f16", split=137)
    np.testing.assert_array_equal(a, c)
