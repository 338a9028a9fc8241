"""Replica logic of bench.py across ranks (CPU, gloo, world size 2): every
rank filters its own image, the job's time is the slowest rank's and its
throughput counts every rank's pixels; the reference arm runs on rank 0
alone. No GPU is involved."""

from __future__ import annotations

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, results) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    elapsed = 10.0 + 5.0 * rank  # rank 1 is the slower replica
    slowest = bench.max_over_ranks(elapsed, dist, "cpu")
    value = bench.replica_throughput(world, pixels=1_000_000, steps=4, seconds=slowest)
    results[rank] = (slowest, value)
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_throughput() -> None:
    world, port = 2, _free_port()
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    mp.start_processes(_worker, args=(world, port, results), nprocs=world, join=True, start_method="spawn")
    assert dict(results) == {0: (15.0, 2 * 1_000_000 * 4 / 15.0 / 1e6), 1: (15.0, 2 * 1_000_000 * 4 / 15.0 / 1e6)}


def test_single_process_has_no_reduction() -> None:
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.replica_throughput(1, 100, 2, 1.0) == 200 / 1e6


@pytest.mark.timeout(300)
def test_reference_arm_runs_on_rank_zero_only(tmp_path) -> None:
    """Under torchrun with two ranks, `--impl reference` prints one line
    (rank 0) and the other rank exits 0 without work."""
    pytest.importorskip("torch.distributed.run")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--workload", "nanmedian_direct_3x3_2048_f32", "--gpus", "2",
           "--steps", "1", "--warmup", "3"]
    proc = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=280)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [line for line in proc.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
