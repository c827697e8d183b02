"""Multi-rank host logic of the benchmark, on CPU with the gloo backend (world size 2).

A single traversal does not shard (every round exchanges the frontier), so N GPUs run N independent
replicas; the whole-job figure is the sum of the replicas' work over the slowest replica's time.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms, edges = bench.reduce_job(10.0 + rank, 1000.0 * (rank + 1), world, "cpu")
    q.put((rank, ms, edges))
    dist.destroy_process_group()


def test_reduce_job_two_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for _, ms, edges in got:
        assert ms == 11.0 and edges == 3000.0


def test_reduce_job_single_rank_is_identity():
    import bench

    assert bench.reduce_job(5.0, 7.0, 1, "cpu") == (5.0, 7.0)


def test_shard_queries_cover_and_balance():
    """The batch's static partition: every query exactly once, deterministic, largest-first balance."""
    import numpy as np

    import eegraph_gb300 as E

    rng = np.random.default_rng(7)
    costs = (2 ** rng.uniform(10, 25, 1151)).tolist()
    for world in (1, 2, 4, 8):
        shards = E.shard_queries(costs, world)
        flat = sorted(i for sh in shards for i in sh)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in sh) for sh in shards]
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-6  # LPT bound
        assert shards == E.shard_queries(costs, world)  # every rank gets the same answer
        assert all(sh == sorted(sh) for sh in shards)


def _shard_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import eegraph_gb300 as E

    costs = [float((i * 7919) % 1000 + 1) for i in range(300)]
    mine = E.shard_queries(costs, world)[rank]
    got = [None] * world
    dist.all_gather_object(got, mine)
    # job figures as the batch bench reduces them: slowest rank's time, summed queries
    ms, nq = bench.reduce_job(5.0 + rank, float(len(mine)), world, "cpu")
    q.put((rank, got, ms, nq))
    dist.destroy_process_group()


def test_shards_across_two_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_shard_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = [q.get(timeout=10) for _ in range(world)]
    for rank, got, ms, nq in res:
        flat = sorted(i for sh in got for i in sh)
        assert flat == list(range(300))  # disjoint cover, agreed without exchanging the partition
        assert ms == 6.0 and nq == 300.0


def test_shard_columns():
    import eegraph_gb300 as E

    for C in (1, 2, 31, 64):
        for world in (1, 2, 3, 4, 8):
            sh = E.shard_columns(C, world)
            assert len(sh) == world
            assert [c for s in sh for c in s] == list(range(C))  # contiguous, in order
            sizes = [len(s) for s in sh]
            assert max(sizes) - min(sizes) <= 1
