"""The multi-rank (replicas) path of bench.py on CPU with torch.distributed's gloo backend,
world_size 2: the whole-job rate uses the slowest rank's time, every rank agrees on it, and the
reference arm does its work on rank 0 only."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms_local = 100.0 if rank == 0 else 250.0
    rate, ms = bench.job_rate(1000, ms_local, world)
    dist.barrier()
    # the reference arm returns 0 without work on ranks other than 0
    class A:
        pass

    ref_rc = bench.run_reference(A(), rank, world) if rank != 0 else 0
    out[rank] = (rate, ms, ref_rc)
    dist.destroy_process_group()


def test_job_rate_max_over_ranks():
    world = 2
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
    for r in range(world):
        rate, ms, ref_rc = out[r]
        assert ms == 250.0  # the slowest rank
        assert rate == pytest.approx(world * 1000 / 0.25)
        assert ref_rc == 0
