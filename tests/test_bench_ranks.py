"""CPU tests of bench.py's multi-rank host logic (replicas: one process per
GPU, no data-path collective): two `gloo` ranks agree on the slowest rank's
time, the whole-job throughput counts every replica, and the reference arm
runs on rank 0 only."""

from __future__ import annotations

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(dist, 1.5 + rank)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    world = 2
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_rank_and_job_throughput():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(None, 3.25) == 3.25
    flops = bench.qr_flops(16384, 8192)
    one = bench.job_tflops(1, flops, 444.0)
    assert abs(one - flops / 0.444 / 1e12) < 1e-9
    assert abs(bench.job_tflops(4, flops, 444.0) - 4 * one) < 1e-9  # weak scaling: N replicas


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""  # only rank 0 prints the line
