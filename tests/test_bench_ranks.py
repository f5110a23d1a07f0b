"""bench.py's multi-rank host logic on CPU: N independent replicas (no collective on the
data path), timed as the slowest rank, reported as the whole job's throughput; and the
reference arm's rank handling (rank 0 alone runs and prints)."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = 10.0 * (rank + 1)  # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms, "cpu")
        q.put((rank, slowest, bench.job_rate(1000, 5, world, slowest)))
    finally:
        dist.destroy_process_group()


def test_replicas_report_slowest_rank_and_whole_job_rate():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest time (20 ms) and the job's rate: 2 ranks x 5 steps x 1000
    # units in 20 ms
    assert got == [(0, 20.0, 500000.0), (1, 20.0, 500000.0)]


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.job_rate(10, 2, 1, 4.0) == 5000.0


def _run_reference_arm(rank: int) -> subprocess.CompletedProcess:
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--small", "--steps", "1", "--warmup", "0", "--gpus", "2"]
    return subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_other_ranks_exit_quietly():
    r = _run_reference_arm(1)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_rank0_prints_the_contract_line():
    r = _run_reference_arm(0)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["value"] > 0
