"""Replica sharding across ranks on CPU (gloo, world size 2): disjoint view
shards covering every view, and the job time as the slowest rank's with the
units summed -- the only cross-rank step of the multi-GPU benchmark."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from xray_projection_render_gb300.sharding import job_time, shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        views = [(2.0 * k, 90.0) for k in range(11)]
        mine = shard(views, rank, world)
        t, u = job_time(0.5 + rank, 100.0 * len(mine))
        q.put((rank, mine, t, u))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_and_job_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out.sort()
    allv = [v for _, mine, _, _ in out for v in mine]
    assert sorted(allv) == sorted((2.0 * k, 90.0) for k in range(11))
    assert len(set(allv)) == len(allv)
    for _, _, t, u in out:
        assert t == 1.5            # slowest rank
        assert u == 100.0 * 11     # every view once


def test_shard_single_rank_and_errors():
    assert shard([1, 2, 3], 0, 1) == [1, 2, 3]
    assert shard(range(5), 1, 2) == [1, 3]
    with pytest.raises(ValueError):
        shard([1], 2, 2)
    assert job_time(2.0, 7.0) == (2.0, 7.0)
