"""Replicas-only multi-GPU host logic, world_size 2 over gloo on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from nr_gpu_ldpc_gb300.replicas import max_over_ranks, reduce_counts, shard


def test_shard_covers_batch_exactly():
    for n in (0, 1, 7, 4096, 8193):
        for world in (1, 2, 3, 8):
            spans = [shard(n, world, r) for r in range(world)]
            assert spans[0][0] == 0
            for (s0, c0), (s1, _) in zip(spans, spans[1:]):
                assert s0 + c0 == s1
            assert sum(c for _, c in spans) == n
            assert max(c for _, c in spans) - min(c for _, c in spans) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        start, count = shard(1001, world, rank)
        counts = reduce_counts([count, rank + 1, 10 * (rank + 1), 1])
        t = max_over_ranks(1.5 + rank)
        out.put((rank, start, count, counts.tolist(), t))
    finally:
        dist.destroy_process_group()


def test_two_rank_reductions_over_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1:3] for r in res] == [(0, 501), (501, 500)]
    for r in res:
        assert r[3] == [1001, 3, 30, 2]
        assert r[4] == 2.5
