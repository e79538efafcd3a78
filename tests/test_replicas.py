"""Replicas across processes (behf.replicas), on CPU with two gloo ranks: the shot partition, the maximum of the
timed regions and the sum of the gradients -- the only exchanges of the multi-GPU path, which runs independent
replicas or shots and has no collective on the data path."""
from __future__ import annotations

import os

import numpy as np
import pytest

from behf import replicas


def test_shard_partitions_every_shot_once():
    for items in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(items, r, world) for r in range(world)]
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(items))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_single_process_is_identity():
    a = np.arange(6.0).reshape(2, 3)
    assert replicas.max_over_ranks(3.5) == 3.5
    out = replicas.sum_over_ranks(a)
    np.testing.assert_array_equal(out, a)
    assert out is not a


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(5, rank, world)
        slowest = replicas.max_over_ranks(1.0 + rank)
        g = np.full((2, 3), float(rank + 1)) * np.arange(6.0).reshape(2, 3)
        total = replicas.sum_over_ranks(g)
        q.put((rank, mine, slowest, total.tolist()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = (np.arange(6.0).reshape(2, 3) * 3.0).tolist()
    assert res[0][1] == [0, 2, 4] and res[1][1] == [1, 3]
    for _, _, slowest, total in res:
        assert slowest == 2.0
        assert total == expect
