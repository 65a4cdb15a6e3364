"""World sharding across ranks, exercised with 2 gloo processes on the CPU."""
import os
import socket

import pytest

from dbox_gb300 import dist


def test_world_range_partitions():
    for n in (1, 7, 4096, 4097):
        for ws in (1, 2, 3, 8):
            ranges = [dist.world_range(n, r, ws) for r in range(ws)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world_size, port, out):
    import numpy as np
    import torch.distributed as tdist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world_size)
    from dbox_gb300 import scenes
    start, stop = dist.world_range(10, rank, world_size)
    seed = dist.rank_seed(3, rank)
    worlds = scenes.batch(n_worlds=stop - start, seed=seed, lo=8, hi=32)
    local_bodies = sum(scenes.dynamic_body_count(s) for s in worlds)
    elapsed = 1.0 + rank
    t = dist.max_over_ranks(elapsed)
    import torch
    total = torch.tensor([local_bodies], dtype=torch.int64)
    tdist.all_reduce(total)
    out.put((rank, start, stop, t, int(total.item()), local_bodies))
    tdist.destroy_process_group()


def test_two_rank_gloo_sharding():
    import torch.multiprocessing as tmp
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1:3] for r in res] == [(0, 5), (5, 10)]
    assert all(r[3] == 2.0 for r in res)                     # max over ranks
    assert res[0][4] == res[1][4] == res[0][5] + res[1][5]   # body totals agree across ranks
