"""Replica bookkeeping across processes (gloo, world size 2, CPU only)."""

import os
import socket

import pytest

from bone_morphometry_gb300.replicas import shard


def test_shard_partition_and_balance():
    sizes = [5, 100, 7, 64, 64, 3, 250, 1, 80, 80]
    for world in (1, 2, 3, 4):
        parts = [shard(sizes, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, q):
    import torch.distributed as dist

    from bone_morphometry_gb300.replicas import gather_to_rank0, max_over_ranks, shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard(sizes, world, rank)
    t = max_over_ranks(float(10 + rank))
    res = gather_to_rank0((rank, mine))
    dist.barrier()
    if rank == 0:
        q.put((t, res))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp

    sizes = [9, 4, 7, 1, 3, 8]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    t, res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert t == 11.0
    got = dict(res)
    assert sorted(got[0] + got[1]) == list(range(len(sizes)))
    assert got[0] == shard(sizes, 2, 0) and got[1] == shard(sizes, 2, 1)
