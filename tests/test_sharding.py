"""Frames shard across ranks without exchange; the job time is the slowest
rank's.  Two gloo ranks on CPU (no GPU involved)."""
import os
import socket

import numpy as np


def test_shard_frames_partition():
    from pycpet_gb300.sharding import shard_frames

    costs = np.random.default_rng(0).integers(1, 100, 37)
    parts = [shard_frames(costs, r, 4) for r in range(4)]
    allidx = sorted(i for p in parts for i in p)
    assert allidx == list(range(37))                       # every frame exactly once
    loads = [costs[p].sum() for p in parts]
    assert max(loads) - min(loads) <= costs.max()          # LPT balance bound
    assert shard_frames(costs, 0, 1) == list(range(37))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, q):
    import torch.distributed as dist
    from pycpet_gb300.sharding import max_over_ranks, shard_frames, sum_over_ranks

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard_frames(costs, rank, world)
    t = 1.0 + rank            # this rank's "time"
    q.put((rank, mine, max_over_ranks(t), sum_over_ranks(len(mine))))
    dist.destroy_process_group()


def test_two_rank_gloo():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    costs = np.arange(1, 11, dtype=np.float64)
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, t0, n0), (r1, m1, t1, n1) = out
    assert sorted(m0 + m1) == list(range(10)) and not set(m0) & set(m1)
    assert t0 == t1 == 2.0                       # max over ranks
    assert n0 == n1 == 10                        # all frames counted once
