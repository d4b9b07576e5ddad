"""Job partition of batched LUT builds over ranks: two gloo ranks on CPU
(the multi-GPU path shards jobs with no data exchange)."""

from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import sys

    import torch
    import torch.distributed as dist

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "planet-real-time-render_gb300"))
    from planet_renderer_gb300.atmosphere.batch import partition_jobs
    from planet_renderer_gb300.atmosphere.workloads import batched_lut_jobs, batched_lut_sets

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    jobs = batched_lut_jobs(seed=5, snapshots=8, cameras=4)
    cfgs = [c for c, _ in batched_lut_sets()]
    mine = partition_jobs(jobs, cfgs, world, rank)
    load = sum(jobs[i].samples(cfgs[jobs[i].param_set]) for i in mine)
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, load))
    if rank == 0:
        out.put((gathered, len(jobs)))
    dist.destroy_process_group()


def test_partition_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered, n = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    idx = sorted(i for part, _ in gathered for i in part)
    assert idx == list(range(n))  # every job exactly once
    loads = [load for _, load in gathered]
    assert max(loads) - min(loads) <= 0.02 * sum(loads)


def test_partition_rejects_bad_rank():
    from planet_renderer_gb300.atmosphere.batch import partition_jobs

    with pytest.raises(ValueError):
        partition_jobs([], [], 2, 2)
