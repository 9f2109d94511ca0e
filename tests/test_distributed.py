"""Multi-rank host logic on CPU with gloo, world size 2 (every GPU machine in this
run has one GPU): sharding covers each system once, timing takes the max over
ranks, and per-rank partial solves (the oracle stands in for the device solve)
assemble to the full batch."""
import os
import socket

import numpy as np
import pytest

from tridiagonalsolvers_gb300.distributed import shard_range


@pytest.mark.parametrize("m", [0, 1, 7, 65536, 100001])
@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shard_range_partitions_every_system_once(m, world):
    seen = []
    for r in range(world):
        a, b = shard_range(m, r, world)
        assert 0 <= a <= b <= m
        seen.extend(range(a, b))
    assert seen == list(range(m))
    sizes = [shard_range(m, r, world)[1] - shard_range(m, r, world)[0] for r in range(world)]
    assert max(sizes) - min(sizes) <= 1


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import torch

        from oracle import gold
        from tridiagonalsolvers_gb300 import workloads
        from tridiagonalsolvers_gb300.distributed import barrier, max_over_ranks

        m, n = 37, 64
        a, b, c, d = workloads.dominant(m, n, seed=11)
        lo, hi = shard_range(m, rank, world)
        x = gold.serial_many(a[lo:hi], b[lo:hi], c[lo:hi], d[lo:hi])
        barrier()
        t = max_over_ranks(1.0 + rank)
        parts = [None] * world
        dist.all_gather_object(parts, (lo, hi, x))
        if rank == 0:
            full = np.zeros((m, n), np.float32)
            for plo, phi, px in parts:
                full[plo:phi] = px
            q.put((t, float(np.abs(full - gold.serial_many(a, b, c, d)).max())))
        barrier()
        del torch
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_time_and_gather():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    t, err = q.get(timeout=10)
    assert t == 2.0  # max over ranks of 1 + rank
    assert err == 0.0
