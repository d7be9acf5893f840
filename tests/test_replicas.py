"""Replica path with world_size 2 on CPU (gloo): disjoint shards covering all
units, and max-over-ranks timing aggregation."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "concrete-fft_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from concrete_fft import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s, e = replicas.shard(8193, rank, world)
        slowest = replicas.max_over_ranks(1.0 + rank)
        rate = replicas.aggregate_rate(100, 1.0 + rank)
        dist.barrier()
        q.put((rank, s, e, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
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
    res = sorted(q.get(timeout=5) for _ in range(2))
    (_, s0, e0, m0, r0), (_, s1, e1, m1, r1) = res
    assert (s0, e0, s1, e1) == (0, 4097, 4097, 8193)  # disjoint, covering, balanced
    assert m0 == m1 == 2.0                             # max over ranks
    assert r0 == r1 == pytest.approx(2 * 100 / 2.0)    # whole-job rate uses the slowest rank


def test_shard_single_rank():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "concrete-fft_gb300"))
    from concrete_fft import replicas
    assert replicas.shard(10, 0, 1) == (0, 10)
    assert [replicas.shard(10, r, 3) for r in range(3)] == [(0, 4), (4, 7), (7, 10)]
