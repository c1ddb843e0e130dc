"""The several-GPU host path without GPUs: two ranks over gloo (127.0.0.1).
The job's time is the slowest rank's; basin shards cover every cell once, and
each shard run alone gives the bits of the whole-region run for its cells --
the daily step has no exchange between drainage basins, so the ranks need no
collective in the data path."""
import os
import socket

import numpy as np


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from watergap2_gb300 import replicas
    from watergap2_gb300 import synthetic as sy
    seconds = replicas.job_seconds(1.0 + rank, dist)
    region = sy.region_small_swb(seed=12)
    nd = 25
    P, T, S = sy.forcing(region, nd, doy0=100)
    shards = replicas.shard_basins(region, world)
    sub, src = replicas.basin_region(region, shards[rank])
    q, _ = oracle.Oracle(sub).run(100, P[:, src], T[:, src], S[:, src], discharge=True)
    got = [None] * world
    dist.all_gather_object(got, (src, q, int(sub.ncell)))
    if rank == 0:
        queue.put((seconds, got))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_time_and_basin_shards():
    import torch.multiprocessing as mp
    import oracle
    from watergap2_gb300 import replicas
    from watergap2_gb300 import synthetic as sy
    oracle.build()
    ctx = mp.get_context("spawn")
    queue = ctx.SimpleQueue()
    procs = mp.spawn(_worker, args=(2, _free_port(), queue), nprocs=2, join=False)
    seconds, got = queue.get()          # before joining: rank 0 blocks on the pipe until read
    procs.join()
    assert seconds == 2.0                                     # the slower rank's time
    assert replicas.whole_job_value(100.0, 2, seconds) == 100.0
    region = sy.region_small_swb(seed=12)
    nd = 25
    P, T, S = sy.forcing(region, nd, doy0=100)
    q_full, _ = oracle.Oracle(region).run(100, P, T, S, discharge=True)
    cells = np.concatenate([g[0] for g in got])
    assert np.array_equal(np.sort(cells), np.arange(region.ncell))   # every cell in exactly one shard
    sizes = [g[2] for g in got]
    assert max(sizes) - min(sizes) <= max(np.bincount(replicas.basin_of(region)))   # LPT balance
    for src, q, _ in got:
        assert np.array_equal(q, q_full[:, src])
