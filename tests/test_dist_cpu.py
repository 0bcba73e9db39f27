"""Multi-rank plumbing of bench.py on CPU ranks (gloo, world size 2):
replicas are independent, time is the max over ranks, work the sum, and a
batched workload's instances are split so that every instance runs on
exactly one rank."""
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


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out = {}
    for name in ("c4", "c5", "rl_batch16", "c3_dsm"):
        mine = bench.shard(bench.workload(name), name, rank, world)
        pts = sum(c.points for c in mine)
        names = [c.name for c in mine]
        gathered = [None] * world
        dist.all_gather_object(gathered, names)
        _, total = bench.reduce_max_sum(dist, 1.0, float(pts))
        out[name] = (gathered, total, [c.seed for c in mine], bench.scaling_of(name, world))
    q.put((rank, out))
    dist.destroy_process_group()


def test_instances_are_sharded_once_over_two_ranks():
    import bench
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() + 500) % 1000
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    for name in ("c4", "c5", "rl_batch16"):
        full = bench.workload(name)
        gathered, total, _, scaling = res[0][name]
        assigned = [n for per_rank in gathered for n in per_rank]
        assert sorted(assigned) == sorted(c.name for c in full), name      # each instance exactly once
        assert all(len(g) > 0 for g in gathered), name
        assert total == sum(c.points for c in full), name                  # work sums to the whole job
        assert scaling == "strong"
    # a single-channel workload: one replica per rank, each with its own seed
    g0, total, seeds0, scaling = res[0]["c3_dsm"]
    _, _, seeds1, _ = res[1]["c3_dsm"]
    assert len(g0) == 2 and all(len(g) == 1 for g in g0) and g0[0] != g0[1]
    assert seeds0 != seeds1 and scaling == "weak"
    assert total == 2 * bench.workload("c3_dsm")[0].points
