"""Multi-rank host logic (exanbody_gb300/replicas.py) with world_size 2 on CPU
(gloo): max-over-ranks timing, whole-job rate, sharding, gathered latencies."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from exanbody_gb300 import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = replicas.dist_env()
        assert (r, w, lr) == (rank, world, rank)
        slowest = replicas.max_over_ranks(10.0 + rank)
        items = list(range(11))
        mine = replicas.shard(items, rank, world)
        lat = replicas.gather_values(np.arange(len(mine), dtype=np.float64) + 100 * rank)
        out.put((rank, slowest, mine, lat.tolist()))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, m0, l0), (r1, s1, m1, l1) = res
    assert s0 == s1 == 11.0  # the slowest rank's time on every rank
    assert sorted(m0 + m1) == list(range(11)) and not set(m0) & set(m1)
    assert abs(len(m0) - len(m1)) <= 1
    want = list(np.arange(len(m0)) + 0.0) + list(np.arange(len(m1)) + 100.0)
    assert l0 == l1 == want
    from exanbody_gb300 import replicas
    assert replicas.whole_job_rate(4_000_000, 100, 0.5, 2) == 1.6e9
