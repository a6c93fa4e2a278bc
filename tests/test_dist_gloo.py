"""Replicas across ranks (CPU, gloo, world size 2): the aggregation bench.py uses for N GPUs.

The frame pipeline has no cross-GPU exchange, so N GPUs run N independent
replicas; the only collective is the max over ranks of the timed region.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = [40.0, 55.0][rank]            # the replicas' own timed regions
    job = bench._max_over_ranks(dist, local_ms, "cpu")
    out[rank] = (job, bench.whole_job_ms_per_frame(job, 32, world))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (55.0, 55.0 / (32 * 2))
