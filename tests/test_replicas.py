"""The multi-GPU path's host logic with two gloo ranks on the CPU: the replica run's
barrier, slowest-rank time and summed units, and the split of independent items."""

import os
import socket

import pytest
import torch.multiprocessing as mp

from tangerine_gb300.replicas import Replicas, shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    g = Replicas(world, rank, backend="gloo")
    try:
        g.barrier()
        slowest = g.max(1.5 + rank)             # rank 1 is the slower one
        units = g.sum(100 * (rank + 1))
        mine = shard(list(range(11)), rank, world)
        out.put((rank, slowest, units, mine))
        g.barrier()
    finally:
        g.close()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.5, 2.5]
    assert [g[2] for g in got] == [300.0, 300.0]
    a, b = got[0][3], got[1][3]
    assert not set(a) & set(b) and sorted(a + b) == list(range(11))


def test_single_rank_needs_no_group():
    g = Replicas(1, 0)
    assert g.max(3.0) == 3.0 and g.sum(4.0) == 4.0
    g.barrier()
    g.close()
    with pytest.raises(ValueError):
        shard([1, 2], 2, 2)
