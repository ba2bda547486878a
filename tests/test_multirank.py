"""Multi-rank host logic on CPU with the gloo backend (world size 2).

The step does not shard without a halo exchange, so N GPUs run replicas; batched runs split their
scenes over ranks (mps_cuda_gb300.sharding) and only gather statistics.  This test runs two gloo
ranks that partition a 256-scene batch, check that the union is complete and disjoint, take the
max of per-rank timings (the bench's max-over-ranks rule) and gather per-rank particle totals.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, counts, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mps_cuda_gb300.sharding import partition_scenes
    parts = partition_scenes(counts, world)
    mine = parts[rank]
    load = torch.tensor([sum(counts[i] for i in mine)], dtype=torch.int64)
    loads = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(loads, load)
    t = torch.tensor([1.0 + rank], dtype=torch.float64)  # per-rank "elapsed ms"
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    flags = torch.zeros(len(counts), dtype=torch.int32)
    flags[mine] = 1
    dist.all_reduce(flags)
    if rank == 0:
        q.put((int(sum(x.item() for x in loads)), float(t.item()), flags.tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_scene_partition():
    import numpy as np
    rng = np.random.default_rng(1)
    counts = [int(c) for c in np.exp(rng.uniform(np.log(2000), np.log(64000), 256))]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, counts, q)) for r in range(2)]
    for p in procs:
        p.start()
    total, tmax, flags = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert total == sum(counts)
    assert tmax == 2.0
    assert flags == [1] * 256  # every scene on exactly one rank
