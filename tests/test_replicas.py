"""Replicas on several GPUs (bench.py under torchrun): the job's time is the slowest rank's
and the throughput counts every rank's work.  Two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 * (rank + 1)                       # rank 1 is the slower replica
    job_ms = bench.max_over_ranks(ms, world, device="cpu")
    out[rank] = (job_ms, bench.job_throughput(1000, job_ms, world))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_time():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        job_ms, value = out[r]
        assert job_ms == 20.0
        assert value == pytest.approx(2 * 1000 / 0.020)


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.job_throughput(500, 12.5, 1) == pytest.approx(40000.0)
