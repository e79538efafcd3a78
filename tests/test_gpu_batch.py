"""Autotuner and batched shots through the C ABI: the tuned z-chunk length and the batched (overlapping
streams) execution change no result bit."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

import behf
from behf import problems as P

pytestmark = pytest.mark.gpu


def shot(i, n=48, nt=60):
    p = P.small64(n=n, nt=nt, radius=4, cpml=6)
    c = n // 2
    return dataclasses.replace(p, src=(c - 6 + 4 * i, c, c - 3 + 2 * i))


def test_autotune_keeps_results(behf_lib):
    p = shot(0, n=56)
    ref = behf.solver_for(p, precision="f16")
    ref.run(p.nt)
    a = ref.seismograms()
    ref.close()
    s = behf.solver_for(p, precision="f16")
    z, ms = s.autotune(2)
    assert z >= 0 and ms > 0
    assert s.info()["step"] == 0
    s.run(p.nt)
    b = s.seismograms()
    s.close()
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("zchunk", [16, 1000])
def test_zchunk_option_bitwise(behf_lib, zchunk):
    p = shot(1, n=56)
    outs = []
    for z in (0, zchunk):
        s = behf.solver_for(p, precision="f32")
        s.set_option(behf.OPT_ZCHUNK, z)
        s.run(p.nt)
        outs.append(s.seismograms())
        s.close()
    np.testing.assert_array_equal(outs[0], outs[1])


def test_run_batch_matches_sequential(behf_lib):
    probs = [shot(i) for i in range(3)]
    precs = ["f16", "f32", "bf16"]
    seq = []
    for p, pr in zip(probs, precs):
        s = behf.solver_for(p, precision=pr)
        s.run(p.nt)
        seq.append(s.seismograms())
        s.close()
    solvers = [behf.solver_for(p, precision=pr) for p, pr in zip(probs, precs)]
    behf.run_batch(solvers, probs[0].nt)
    for s, ref in zip(solvers, seq):
        np.testing.assert_array_equal(s.seismograms(), ref)
        s.close()


@pytest.mark.parametrize("precision", ["f16", "bf16", "f32"])
def test_run_batch_same_grid_in_two_calls(behf_lib, precision):
    # three shots of one grid: different source kinds and positions, a layered medium for one, stochastic
    # rounding of the stored fields for another (16-bit kinds); batched in two calls (40 + 21 steps: graph
    # chunks of 16 and remainders), against each shot alone
    kinds = ["explosive", "pressure", "force_z"]
    probs = [dataclasses.replace(shot(i, nt=61), src_kind=kinds[i]) for i in range(3)]
    probs[2] = dataclasses.replace(probs[2], mod=P.layered((48, 48, 48), [P.SANDSTONE, P.STIFF], [24]))
    sr = [0, 1 if precision != "f32" else 0, 0]
    seq = []
    for p, r in zip(probs, sr):
        s = behf.solver_for(p, precision=precision, state_rounding=r)
        s.run(p.nt)
        seq.append(s.seismograms())
        s.close()
    solvers = [behf.solver_for(p, precision=precision, state_rounding=r) for p, r in zip(probs, sr)]
    behf.run_batch(solvers, 40)
    behf.run_batch(solvers, 21)
    for s, ref in zip(solvers, seq):
        assert s.info()["step"] == 61
        np.testing.assert_array_equal(s.seismograms(), ref)
        s.close()
