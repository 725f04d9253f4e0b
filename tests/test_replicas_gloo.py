"""The multi-process (replica) path on CPU: world_size 2 with gloo.

The workloads are independent per GPU (replicas; batched problems shard with
no data-path collective), so the only collectives are the barrier and the
max-over-ranks reduction of the timed region, and the problem partition must
be disjoint and complete.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from parla_gb300.drivers.batched import shard_indices
    mine = shard_indices(10, rank, world)
    t = torch.tensor([10.0 + rank], dtype=torch.float64)   # this rank's timed region (ms)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    got = [None] * world
    dist.all_gather_object(got, mine)
    if rank == 0:
        out.put((float(t.item()), got))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_barrier_max_and_shards():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    tmax, shards = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert tmax == 11.0
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(10))
    assert not set(shards[0]) & set(shards[1])


def test_shard_indices_single_process():
    from parla_gb300.drivers.batched import shard_indices
    assert shard_indices(7, 0, 1) == list(range(7))
    parts = [shard_indices(7, r, 3) for r in range(3)]
    assert sorted(i for p in parts for i in p) == list(range(7))
