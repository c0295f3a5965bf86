"""Multi-process path on CPU (gloo, world size 2): ray shards cover the batch
exactly once and the summed counter totals equal a single process's."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from bvhraytracer_gb300.shard import reduce_totals, shard_range


def test_shard_ranges_partition():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            got = [shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [e - b for b, e in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from tests import _scenes as TS
    tris, b, cv = TS.bvh("terrain", 4, 4)
    rays = TS.terrain_case()[1][::16]
    lo, hi = shard_range(rays.shape[0], rank, world)
    r = O.trace_instrumented(cv, rays[lo:hi], shadow=False)
    totals = torch.from_numpy(r["counters"].astype(np.int64).sum(0))
    hist = torch.from_numpy(r["depth_hist"].astype(np.int64).reshape(-1))
    reduce_totals(totals)
    reduce_totals(hist)
    if rank == 0:
        out.put((totals.numpy(), hist.numpy()))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_sum_counters():
    from oracle import oracle as O
    from tests import _scenes as TS
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    totals, hist = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    tris, b, cv = TS.bvh("terrain", 4, 4)
    rays = TS.terrain_case()[1][::16]
    r = O.trace_instrumented(cv, rays, shadow=False)
    assert np.array_equal(totals, r["counters"].astype(np.int64).sum(0))
    assert np.array_equal(hist, r["depth_hist"].astype(np.int64).reshape(-1))
