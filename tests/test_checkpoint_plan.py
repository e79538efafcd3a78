"""The gradient's checkpoint plan (behf_checkpoint_plan, host arithmetic of libbehf.so; no GPU): one level of
round(sqrt(nt)) spacing when it fits, two levels with the inner spacing halved until the cheapest outer spacing
fits, the explicit spacings of BEHF_OPT_CHECKPOINT / BEHF_OPT_CHECKPOINT_OUTER, and the bytes reported."""
from __future__ import annotations

import math

import numpy as np
import pytest

import behf

GB = 10 ** 9


def need(nt, s2, s1, ck, snap, fixed=0):
    nout = -(-nt // s1)
    nin = -(-s1 // s2) if s1 > s2 else 0
    return (nout + nin) * ck + (s2 + 1) * snap + fixed


def search(nt, ck, snap, avail, fixed=0, checkpoint=0):
    """The planner's choice restated: halve the inner spacing until the outer spacing (a multiple k >= 2 of it,
    below 2 nt) that needs the least memory fits."""
    s = checkpoint or max(1, round(math.sqrt(nt)))
    s = min(s, nt)
    if need(nt, s, s, ck, snap, fixed) <= avail:
        return s, s
    s2 = s
    while s2 >= 1:
        cands = [(need(nt, s2, k * s2, ck, snap, fixed), k * s2) for k in range(2, (2 * nt - 1) // s2 + 1)]
        if cands:
            best = min(cands, key=lambda c: c[0])  # first of equal minima, as the planner keeps
            if best[0] <= avail:
                return s2, best[1]
        s2 = 0 if checkpoint else s2 // 2
    return s, s


def test_one_level_when_it_fits():
    # 256^3 FP16, 2000 steps: 45 checkpoints of 0.95 GB and 46 snapshots of 0.44 GB
    inner, outer, nbytes = behf.checkpoint_plan(2000, int(0.95 * GB), int(0.44 * GB), avail=250 * GB)
    assert (inner, outer) == (45, 45)
    assert nbytes == need(2000, 45, 45, int(0.95 * GB), int(0.44 * GB))


def test_two_levels_when_one_does_not_fit():
    # 512^3 FP16, 2000 steps: one level needs 410 GB; with 234 GB the inner spacing halves once
    ck, snap = int(5.55 * GB), int(3.49 * GB)
    assert need(2000, 45, 45, ck, snap) > 234 * GB
    inner, outer, nbytes = behf.checkpoint_plan(2000, ck, snap, avail=234 * GB)
    assert (inner, outer) == (22, 154)
    assert nbytes == need(2000, 22, 154, ck, snap) <= 234 * GB
    # with room for the first inner spacing it keeps it
    inner, outer, nbytes = behf.checkpoint_plan(2000, ck, snap, avail=240 * GB)
    assert inner == 45 and outer % 45 == 0 and outer > 45 and nbytes <= 240 * GB


def test_fixed_inner_spacing_and_nothing_fits():
    ck, snap = int(5.55 * GB), int(3.49 * GB)
    # BEHF_OPT_CHECKPOINT fixes the inner spacing: only its outer spacings are tried
    inner, outer, _ = behf.checkpoint_plan(2000, ck, snap, avail=234 * GB, checkpoint=45)
    assert (inner, outer) == (45, 45)  # 238 GB at best: falls back to one level (its allocation fails loudly)
    inner, outer, _ = behf.checkpoint_plan(2000, ck, snap, avail=1 * GB)
    assert (inner, outer) == (45, 45)


def test_explicit_outer_spacing_and_clamps():
    # outer spacing rounded up to a multiple of the inner one; avail is not consulted
    assert behf.checkpoint_plan(100, 10, 5, avail=0, checkpoint=13, checkpoint_outer=30)[:2] == (13, 39)
    assert behf.checkpoint_plan(100, 10, 5, avail=0, checkpoint=13, checkpoint_outer=5)[:2] == (13, 13)
    # an inner spacing above nt is nt (one segment)
    assert behf.checkpoint_plan(60, 10, 5, avail=10 ** 12, checkpoint=100)[:2] == (60, 60)
    assert behf.checkpoint_plan(1, 10, 5, avail=10 ** 12)[:2] == (1, 1)


def test_invalid_arguments():
    with pytest.raises(behf.BehfError):
        behf.checkpoint_plan(0, 10, 5, avail=100)
    with pytest.raises(behf.BehfError):
        behf.checkpoint_plan(10, 10, 5, avail=100, checkpoint=-1)


def test_matches_the_search_on_random_sizes():
    rng = np.random.default_rng(7)
    for _ in range(300):
        nt = int(rng.integers(1, 5000))
        ck = int(rng.integers(1, 50)) * 10 ** 8
        snap = int(rng.integers(1, 30)) * 10 ** 8
        fixed = int(rng.integers(0, 10)) * 10 ** 6
        fixed_ck = int(rng.choice([0, 0, 0, int(rng.integers(1, 100))]))
        s = fixed_ck or max(1, round(math.sqrt(nt)))
        one = need(nt, min(s, nt), min(s, nt), ck, snap, fixed)
        avail = int(one * rng.uniform(0.05, 1.3))
        inner, outer, nbytes = behf.checkpoint_plan(nt, ck, snap, avail=avail, checkpoint=fixed_ck,
                                                    fixed_bytes=fixed)
        assert (inner, outer) == search(nt, ck, snap, avail, fixed, fixed_ck), (nt, ck, snap, fixed, fixed_ck, avail)
        assert nbytes == need(nt, inner, outer, ck, snap, fixed)
        assert outer % inner == 0 and 1 <= inner <= nt
        if outer > inner:
            assert nbytes <= avail
