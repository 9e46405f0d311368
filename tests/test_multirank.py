"""Multi-GPU host logic on CPU: two gloo ranks.  The path runs as replicas
(one independent job per rank, no data-path collective); the only
cross-rank steps are the max-over-ranks time and, for job lists, a
round-robin shard that must be disjoint and complete."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # slowest rank decides the job-wide time
    t = bench.reduce_max(10.0 + 5.0 * rank)
    # jobs sharded round-robin: gather every rank's ids
    mine = bench.shard(list(range(37)), rank, world)
    sizes = [None] * world
    dist.all_gather_object(sizes, mine)
    q.put((rank, t, sizes))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_reduction_and_shards(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, shards in out:
        assert t == 10.0 + 5.0 * (world - 1)
        flat = sorted(x for sh in shards for x in sh)
        assert flat == list(range(37))
        assert len(set(flat)) == 37
