"""The benchmark's multi-rank plumbing on CPU (gloo, two ranks): replicas on
every rank, the slowest rank's time, the whole-job rate, and the reference
arm under torchrun (rank 0 prints the one line, the other ranks do no work)."""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    slowest = bench.max_over_ranks(10.0 + rank, world)  # rank r took 10 + r ms
    out[rank] = (slowest, bench.replicas_rate(1000, 5, slowest, world))
    dist.destroy_process_group()


def test_slowest_rank_time_and_whole_job_rate_over_two_gloo_ranks():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert out[0] == out[1] == (11.0, 2 * 1000 * 5 / 11e-3)


def test_reference_arm_under_torchrun_prints_one_line_from_rank_zero():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-sample", "24", "--cpu-steps", "1"]
    run = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [line for line in run.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    record = json.loads(lines[0])
    assert record["impl"] == "reference" and record["n_gpus"] == 2 and record["value"] > 0
    assert record["cpu_baseline"]["kind"] == "port" and record["e2e"]["h2d_bytes_per_step"] == 0
