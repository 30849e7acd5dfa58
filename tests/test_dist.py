"""Multi-rank host logic on CPU (gloo, world_size 2): the max-over-ranks
timing reduction bench.py uses for replicas, and the matrix sharding of a
batch (every matrix on exactly one rank, all ranks agreeing)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, nnz, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from edge_loops_gb300.dist import max_over_ranks, shard_matrices
        mx = max_over_ranks(1.5 + rank)  # rank 0: 1.5, rank 1: 2.5
        shards = shard_matrices(nnz, world)
        mine = shards[rank]
        everyone = [None] * world
        dist.all_gather_object(everyone, mine)
        q.put((rank, mx, everyone, shards))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    nnz = [5, 100, 7, 7, 64, 0, 33, 1000, 12, 2]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, nnz, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, everyone, shards in out:
        assert mx == 2.5
        assert everyone == shards  # every rank computed the same assignment
    shards = out[0][3]
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(nnz)))
    loads = [sum(nnz[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(nnz)


def test_single_process_helpers():
    from edge_loops_gb300.dist import max_over_ranks, shard_matrices
    assert max_over_ranks(3.25) == 3.25  # no process group: the value itself
    assert shard_matrices([3, 1, 2], 1) == [[0, 1, 2]]
    assert shard_matrices([], 3) == [[], [], []]
    s = shard_matrices([10, 10, 10, 10], 4)
    assert sorted(len(x) for x in s) == [1, 1, 1, 1]
    with pytest.raises(ValueError):
        shard_matrices([1], 0)
