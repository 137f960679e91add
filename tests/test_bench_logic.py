"""CPU tests of the benchmark's workload definition and its multi-rank
aggregation (world_size 2 over gloo)."""
import os

import numpy as np
import pytest


def test_workload_lengths():
    import bench
    L = bench.workload_lengths()
    assert L[-3:] == [1009, 8191, 65521]
    sm = set(bench.smooth_numbers(64, 65536))
    assert all(n in sm for n in L[:-3]) and len(L) >= 30
    assert all(64 <= n <= 65536 for n in L)
    tot = sum(bench.batch_for(n) * n for n in L)
    assert abs(tot / len(L) - (1 << 24)) < 0.01 * (1 << 24)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 if rank == 0 else 12.5
    v = bench.aggregate(ms, 1e9, world, device=None)
    q.put((rank, v))
    dist.destroy_process_group()


def test_two_rank_aggregation():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    res = dict(q.get() for _ in range(2))
    # max over ranks (12.5 ms), weak scaling: 2 ranks x 1 GB each
    assert res[0] == res[1]
    ms, gbs = res[0]
    assert ms == 12.5 and abs(gbs - 2e9 / 12.5e-3 / 1e9) < 1e-9
