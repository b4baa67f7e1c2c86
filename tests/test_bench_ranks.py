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
    sys.path.insert(0, str(ROOT))
    import bench
    # The reference arm describes the same workload as our line, on the grid it ran.
    assert record["config"] == bench.workload_config(24, 2)
    assert "24x24 grid" in record["cpu_baseline"]["sample"]


def test_summary_carries_every_block_headline():
    sys.path.insert(0, str(ROOT))
    import bench
    roof = {"stage_ms": 7.5, "frac": 0.99, "fp64_nominal": {"frac": 0.83}, "hbm": {"frac": 0.03}}
    line = {"value": 7e8, "e2e": {"value": 6.9e8}, "roofline": roof,
            "fp32": {"value": 2e10, "e2e": {"value": 9e9}, "roofline": dict(roof, hbm={"frac": 0.45})},
            "cpu_baseline": {"value": 4.6e6, "cores": 16},
            "serving": {"mixed_80pct_fp32_rate1000": {"solves_per_s": 200.0, "speedup_vs_serial_fp64": 6.5,
                                                      "tts_p50_s": 0.2, "tts_p99_s": 0.4, "arrival_bound": False,
                                                      "fp32_l1_density_err_vs_fp64_max": 5e-7}}}
    s = bench.summary(line)
    assert s["f64"]["frac_of_nominal"] == 0.83 and s["f32"]["hbm_frac"] == 0.45
    assert s["cpu_baseline"] == {"cell_updates_per_s": 4.6e6, "cores": 16, "f64_e2e_over_cpu": 150.0}
    assert s["serving"]["mixed_80pct_fp32_rate1000"] == [200.0, 6.5, 0.2, 0.4, False]
    assert s["serving_fp32_l1_max"] == 5e-7 and s["serving_fp32_l1_max_unguarded"] is None
