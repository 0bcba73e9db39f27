"""Multi-rank plumbing of bench.py on CPU ranks (gloo, world size 2):
replicas are independent, time is the max over ranks, work the sum."""
import os

import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, w = bench.reduce_max_sum(dist, 10.0 + rank, 1000.0 * (rank + 1))
    bench.barrier(dist)
    q.put((rank, t, w))
    dist.destroy_process_group()


def test_reduce_max_sum_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res == [(0, 11.0, 3000.0), (1, 11.0, 3000.0)]
