#!/usr/bin/env python
"""Benchmark of the fused per-RK-stage isothermal hydro right-hand side on GB300.

Workload (one "step" = one evolve_isothermal cycle: CFL dt + 3 fused RK3
stages): the tanh Kelvin-Helmholtz layer with a tracer, 4096 x 4096 cells,
4 variables (rho, rho vx, rho vy, rho s), PPM4 + Roe, RK3, CFL 0.4, float64
state. The same workload in float32 is reported under "fp32". Synthetic
initial data; the state (537 MB in float64) is larger than the 129 MB L2, so
no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line on rank 0. With N > 1 (torchrun) every rank advances its
own independent copy of the workload (replicas, no collective on the data
path) and the value is the sum over ranks.
"""

import argparse
import ctypes
import csv
import io
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s"
WORKLOAD = "kelvin_helmholtz_tanh 4096x4096, 4 vars, ppm4+roe, rk3, cfl 0.4"
PEAKS = ROOT / "MEASURED_PEAKS.json"
# ncu-measured DRAM bytes per cell for one launch of the fused stage kernel
# (stage 2 of RK3, ppm4+roe, 4 variables), from the capture summarised in
# profiles/; None until such a capture exists for the dtype.
# DRAM bytes (read + write) of one RK3 stage-2 launch at 4096^2, from a one-pass
# ncu capture of this benchmark (dram__bytes_read.sum + dram__bytes_write.sum).
# Thread instructions per cell of the float32 marching stage (ppm4+roe, 4
# variables, packed-pair walk with the row ring): smsp__inst_executed.sum x
# 32 / cells of one launch.
STAGE_INST_PER_CELL_F32 = 125.14e6 * 32 / 3072**2
STAGE_TRAFFIC_BYTES_PER_CELL = {"f64": (1075.99e6 + 509.14e6) / 4096**2, "f32": (552.01e6 + 236.64e6) / 4096**2}


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=("ours", "reference"), default="ours")
    p.add_argument("--n", type=int, default=None, help="grid side (default 4096; 1024 with --sweep)")
    p.add_argument("--no-fp32", action="store_true", help="skip the float32 line")
    p.add_argument("--only-fp32", action="store_true", help="time only the float32 state (profiling)")
    p.add_argument("--cpu-sample", type=int, default=None,
                   help="grid side of the CPU (oracle) run (default: the benchmark grid, --n or 4096)")
    p.add_argument("--cpu-steps", type=int, default=4,
                   help="timed cycles of the CPU run in our line (the reference arm times min(--steps, 8))")
    p.add_argument("--no-patterns", action="store_true",
                   help="skip the batched / serving / precision measurements")
    p.add_argument("--serve-requests", type=int, default=100)
    p.add_argument("--turbulence-t", type=float, default=None,
                   help="instead of the benchmark line: the driven-turbulence configuration on the --n "
                        "grid (default 1024 here) to this end time in float32 and float64, with the "
                        "precision report (L1 error, drift, KE spectrum deviation)")
    p.add_argument("--cs", type=float, default=0.0, help="Smagorinsky constant for --turbulence-t")
    p.add_argument("--average-from", type=float, default=None,
                   help="with --turbulence-t: also compare KE spectra averaged over t = T0, T0+1, ..., end")
    p.add_argument("--chaos-floor", action="store_true",
                   help="with --turbulence-t: add a float64 run from a 1e-12-perturbed density")
    p.add_argument("--ensemble", choices=("all", "kh", "turbulence"), default=None,
                   help="instead of the benchmark line: time --steps batched cycles (after --warmup) of "
                        "the 64-solve float32 ensemble (or its KH / turbulence half) at --tile")
    p.add_argument("--tile", default="58x32", help="tile of --ensemble, e.g. 58x32 or 32x16")
    p.add_argument("--precision-sweep", action="store_true",
                   help="instead of the benchmark line: float32 against float64 L1 density error of every "
                        "problem x reconstruction x Riemann solver on small served grids (one JSON line each)")
    p.add_argument("--precision-tlims", default="0.5,1,1.5,2,2.5,3", help="end times of --precision-sweep")
    p.add_argument("--precision-pairs", default="",
                   help="problem:reconstruction pairs of --precision-sweep, e.g. kh:ppm4,smooth:wenoz (default all)")
    p.add_argument("--serve-stated", type=int, default=None, metavar="N",
                   help="instead of the benchmark line: the stated serving stream (side 64..2048, "
                        "tlim U[0.2, 3]) with N requests at --serve-rate, against serial float64")
    p.add_argument("--serve-rate", type=float, default=1000.0)
    p.add_argument("--sweep", action="store_true",
                   help="instead of the benchmark line: one JSON line per reconstruction x Riemann "
                        "solver x integrator x precision on the --n grid (default 1024 here)")
    return p.parse_args()


# ---------------------------------------------------------------------------
# Distributed plumbing (replicas only).
# ---------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world):
    """The largest of every rank's value (the slowest rank's time)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    device = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_rate(cells_per_step, steps, ms, world):
    """Whole-job cell-updates/s: every rank advances its own replica of
    `cells_per_step` cells `steps` times; `ms` is the slowest rank's time."""
    return world * cells_per_step * steps / (ms * 1e-3)


# ---------------------------------------------------------------------------
# Clock sampling during the timed region.
# ---------------------------------------------------------------------------
QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        if shutil.which("nvidia-smi") is None:
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.handle = open(self.path, "w")
        self.proc = subprocess.Popen(
            ["nvidia-smi", f"--query-gpu={QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
             "-i", str(gpu_index)], stdout=self.handle, stderr=subprocess.DEVNULL)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.handle.close()
        rows = list(csv.reader(io.StringIO(Path(self.path).read_text())))
        os.unlink(self.path)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for row in rows:
            row = [c.strip() for c in row]
            if len(row) < 9:
                continue
            try:
                sm.append(float(row[1]))
                smax.append(float(row[2]))
            except ValueError:
                continue
            for name, flag in zip(names, row[5:9]):
                if flag.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def nvidia_smi_index(local_rank):
    visible = os.environ.get("CUDA_VISIBLE_DEVICES")
    if visible:
        entries = [v for v in visible.split(",") if v.strip()]
        if local_rank < len(entries) and entries[local_rank].strip().isdigit():
            return int(entries[local_rank])
    return local_rank


# ---------------------------------------------------------------------------
# Our arm.
# ---------------------------------------------------------------------------
def fma_peak(torch, _lib, dtype_id, gpu_index=None):
    """Measured FMA throughput of the FP64 or FP32 pipe with every SM busy.

    Sweeps 8/16/32 independent chains per thread at 4 and 8 resident blocks
    of 256 threads per SM and keeps the fastest; with ``gpu_index`` the SM
    clock is sampled meanwhile, so the rate is also stated as FMAs per SM
    per clock cycle. Returns {"tflops", "fma_per_sm_per_clk", "sm_mhz",
    "sms", "trials"}.
    """
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    sink = torch.zeros(sms * 8, dtype=torch.float64, device="cuda")
    stream = _lib.stream_handle()
    rate = 1.2e12 if dtype_id == _lib.JX_F64 else 90e12  # flop/s, to size ~25 ms launches
    sampler = ClockSampler(gpu_index) if gpu_index is not None else None
    trials = []
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for chains in (8, 16, 32):
        for per_sm in (4, 8):
            blocks = sms * per_sm
            iters = max(64, int(0.025 * rate / (2.0 * chains * blocks * 256)))
            _lib.call("jx_probe_fma", dtype_id, blocks, iters, chains, _lib.ptr(sink), stream)
            best = None
            for _ in range(3):
                start.record()
                _lib.call("jx_probe_fma", dtype_id, blocks, iters, chains, _lib.ptr(sink), stream)
                end.record()
                end.synchronize()
                ms = start.elapsed_time(end)
                best = ms if best is None else min(best, ms)
            flops = 2.0 * chains * iters * blocks * 256
            trials.append({"chains": chains, "blocks_per_sm": per_sm, "tflops": round(flops / (best * 1e-3) / 1e12, 4)})
    clocks = sampler.stop() if sampler is not None else {"sm_mhz": None}
    top = max(trials, key=lambda r: r["tflops"])
    mhz = clocks.get("sm_mhz")
    per_clk = top["tflops"] * 1e12 / 2.0 / (sms * mhz * 1e6) if mhz else None
    return {"tflops": top["tflops"], "fma_per_sm_per_clk": None if per_clk is None else round(per_clk, 3),
            "sm_mhz": mhz, "sms": sms, "best": {k: top[k] for k in ("chains", "blocks_per_sm")}, "trials": trials}


def measured_peaks():
    if PEAKS.exists():
        return json.loads(PEAKS.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def flops_per_cell_stage(key):
    table = json.loads((ROOT / "jathenax_gb300" / "flops.json").read_text())["flops_per_cell_stage"]
    return table[key]


def run_precision(torch, _lib, Solve, U0, n, dtype, args, world, clocks=None):
    """Time K steps of the resident solve; time the stage kernel alone; e2e."""
    solve = Solve(U0, 1.0 / n, 1.0 / n, 1.0, 1e-10, "rk3", 0.4, 1e30, 2**31 - 1,
                  reconstruct="ppm4", rsolver="roe", dtype=dtype)
    solve.capture(1)
    for _ in range(args.warmup):
        solve.graph.replay()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    sampler = ClockSampler(clocks) if clocks is not None else None
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        solve.graph.replay()
    end.record()
    torch.cuda.synchronize()
    clock_info = sampler.stop() if sampler is not None else None
    barrier(world)
    ms = max_over_ranks(start.elapsed_time(end), world)
    cells = n * n
    value = replicas_rate(cells, args.steps, ms, world)
    state = solve.state()

    # The dominant kernel alone: stage 2 (blend form) reading A, pointwise S, writing B.
    solve.A.copy_(solve.S)
    reps = max(3, min(20, args.steps))
    solve.enqueue_stage(2, solve.A, solve.S, solve.B)
    torch.cuda.synchronize()
    ks, ke = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ks.record()
    for _ in range(reps):
        solve.enqueue_stage(2, solve.A, solve.S, solve.B)
    ke.record()
    torch.cuda.synchronize()
    stage_ms = ks.elapsed_time(ke) / reps

    # End to end through the public API: each step uploads a state from pinned
    # host memory, advances it one cycle and downloads the result; the uploads
    # and downloads of neighbouring steps overlap the cycles (advance_host_many).
    host_in = solve.S.cpu().pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    e2e_steps = max(2, args.steps)  # as many steps as the device-timed run
    solve.advance_host_many([host_in] * 2, [host_out] * 2)
    torch.cuda.synchronize()
    barrier(world)
    es, ee = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    es.record()
    solve.advance_host_many([host_in] * e2e_steps, [host_out] * e2e_steps)
    ee.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(es.elapsed_time(ee), world)
    state_bytes = host_in.numel() * host_in.element_size()
    tx, ty, smem = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
    _lib.call("jx_tile_info", ctypes.byref(solve.desc), ctypes.byref(tx), ctypes.byref(ty), ctypes.byref(smem))
    return dict(value=value, ms=ms, stage_ms=stage_ms, clocks=clock_info, solve_state=state, tile=(tx.value, ty.value),
                e2e=dict(value=replicas_rate(cells, e2e_steps, e2e_ms, world), unit=METRIC,
                         h2d_bytes_per_step=state_bytes, d2h_bytes_per_step=state_bytes),
                dt=state.dt)


def cpu_baseline_sample(n, steps, procs=None):
    """The float64 oracle (NumPy) on the whole n x n tanh KH grid: one untimed,
    then `steps` timed evolve cycles (dt + 3 RK stages), the grid split into row
    slabs over `spawn`ed processes, one per host core (oracle.slab; bit for bit
    the oracle's whole-grid cycles). The rate is the grid's cell-updates over
    the slowest process's time."""
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    from oracle import slab
    _, seconds, procs = slab.run(kelvin_helmholtz_tanh(n, n), cycles=steps, procs=procs, warm=1)
    return dict(value=n * n * steps / seconds, unit=METRIC, cores=procs, kind="port",
                sample=f"float64 NumPy oracle on the whole kelvin_helmholtz_tanh {n}x{n} grid, {steps} full "
                       f"RK3 cycles (dt + 3 stages) after 1 untimed, in {procs} row slabs of about "
                       f"{n // procs} rows (one process per host core, 3 halo rows a stage)",
                seconds=round(seconds, 2))


def workload_config(n, world):
    """The benchmark workload, the same in both arms' lines."""
    return {"workload": WORKLOAD.replace("4096x4096", f"{n}x{n}"), "nx": n, "ny": n, "nvar": 4,
            "reconstruct": "ppm4", "rsolver": "roe", "integrator": "rk3", "cfl": 0.4,
            "step": "one evolve cycle: CFL dt + 3 RK stages",
            "l2": f"state {n * n * 4 * 8 / 1e6:.0f} MB" + (" > 129 MB L2 (no flush needed)"
                                                           if n * n * 4 * 8 > 129e6 else ""),
            "parallelism": f"replicas x{world}"}


def bench_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    from jathenax_gb300 import _lib
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    from jathenax_gb300.solver import Solve

    n = args.n
    U0 = torch.as_tensor(kelvin_helmholtz_tanh(n, n), device="cuda")
    peaks, peak_kind = measured_peaks()
    if args.only_fp32:
        r32 = run_precision(torch, _lib, Solve, U0, n, torch.float32, args, world)
        return {"metric": METRIC, "value": round(r32["value"], 1), "unit": METRIC, "dtype": "f32",
                "ms_per_step": round(r32["ms"] / args.steps, 4), "stage_ms": r32["stage_ms"]}
    gpu = nvidia_smi_index(local)
    probe64 = fma_peak(torch, _lib, _lib.JX_F64, gpu)
    probe32 = fma_peak(torch, _lib, _lib.JX_F32, gpu)
    r64 = run_precision(torch, _lib, Solve, U0, n, torch.float64, args, world,
                        clocks=nvidia_smi_index(local))
    r32 = None if args.no_fp32 else run_precision(torch, _lib, Solve, U0, n, torch.float32, args, world)

    cells = n * n
    fpcs = flops_per_cell_stage("ppm4/roe/nvar4")
    nvar, w64 = 4, 8

    def roofline(res, w, probe, key):
        peak_tflops = probe["tflops"]
        flops = cells * fpcs / (res["stage_ms"] * 1e-3) / 1e12
        stage_bytes = 3 * w * nvar * cells  # stage >= 2: read U and V, write U
        gbs = stage_bytes / (res["stage_ms"] * 1e-3) / 1e9
        traffic = STAGE_TRAFFIC_BYTES_PER_CELL[key]
        hbm_peak = peaks["hbm_gbs"]
        compute_frac = flops / peak_tflops
        hbm_frac = gbs / hbm_peak
        bound = "fp64" if key == "f64" else ("fp32" if compute_frac >= hbm_frac else "hbm")
        tx, ty = res["tile"]
        if w == 4 and tx == 58:
            # float32, two columns per lane: the packed-pair walk; from 24 rows the
            # row-ring kernel at 112 registers with the x sweep first
            kernel = (f"stage_kernel_march_pk_x<roe,4,blend> (PPM4, row ring, x sweep first, 112 registers, packed pairs"
                      if ty >= 24 else "stage_kernel_march_pk<ppm4,roe,4,blend> (packed pairs")
        else:
            family = "stage_kernel_march" if tx in (26, 58, 90) else "stage_kernel_fast"
            kernel = f"{family}<{'double' if w == 8 else 'float'},ppm4,roe,4> ("
        out = {"kernel": f"{kernel}{', ' if kernel[-1] != '(' else ''}RK3 stage 2, tile {tx}x{ty})",
               "bound": bound, "achieved": round(flops, 4), "peak": round(peak_tflops, 4),
               "unit": "TFLOP/s", "frac": round(compute_frac, 4),
               "peak_source": f"{key.upper()} FMA pipe measured live by jx_probe_fma",
               "flops_per_cell_stage": fpcs,
               "traffic": None if traffic is None else traffic * cells,
               "stage_ms": round(res["stage_ms"], 4),
               "hbm": {"achieved": round(gbs, 1), "peak": hbm_peak, "unit": "GB/s",
                       "frac": round(hbm_frac, 4), "peak_source": f"hbm_gbs of {peak_kind}",
                       "bytes_per_launch": stage_bytes}}
        out["probe"] = {k: probe[k] for k in ("fma_per_sm_per_clk", "sm_mhz", "sms", "best")}
        if key == "f64":
            # The same work against GB300's nominal float64 rate, 2 DFMA per SM
            # per clock at the SM clock sampled during the timed steps.
            mhz = (res.get("clocks") or {}).get("sm_mhz") or probe["sm_mhz"]
            if mhz:
                nominal = 2 * 2 * probe["sms"] * mhz * 1e6 / 1e12
                out["fp64_nominal"] = {"peak": round(nominal, 4), "unit": "TFLOP/s", "frac": round(flops / nominal, 4),
                                       "peak_source": f"2 DFMA/SM/clk x {probe['sms']} SMs x {mhz:.0f} MHz"}
        if key == "f32":
            # The float32 marching stage is bound by instruction issue: its
            # executed instructions per cell (ncu, 3072² case) over the issue
            # rate of every scheduler (4 per SM, one warp instruction per clock).
            mhz = (res.get("clocks") or {}).get("sm_mhz") or probe["sm_mhz"]
            if mhz:
                bound_ms = cells * STAGE_INST_PER_CELL_F32 / 32 / (probe["sms"] * 4 * mhz * 1e6) * 1e3
                out["issue"] = {"thread_instructions_per_cell": round(STAGE_INST_PER_CELL_F32, 1), "bound_ms": round(bound_ms, 4),
                                "frac": round(bound_ms / res["stage_ms"], 4),
                                "source": "smsp__inst_executed.sum of one stage launch (ncu, 3072x3072)"}
        if bound == "hbm":
            out.update(achieved=round(gbs, 1), peak=hbm_peak, unit="GB/s", frac=round(hbm_frac, 4),
                       peak_source=f"hbm_gbs of {peak_kind}")
        return out

    line = {
        "metric": METRIC, "value": round(r64["value"], 1), "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(r64["ms"] / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, world),
        "roofline": roofline(r64, w64, probe64, "f64"),
        "e2e": r64["e2e"],
        "gpu_launches": 4 * args.steps,  # per step: begin-step + 3 stage kernels
        "clocks": r64["clocks"],
    }
    if r32 is not None:
        line["fp32"] = {"value": round(r32["value"], 1), "unit": METRIC,
                        "ms_per_step": round(r32["ms"] / args.steps, 4), "dtype": "f32",
                        "roofline": roofline(r32, 4, probe32, "f32"), "e2e": r32["e2e"],
                        "gpu_launches": 4 * args.steps}
    if rank == 0 and world == 1 and args.cpu_steps > 0:
        line["cpu_baseline"] = cpu_baseline_sample(args.cpu_sample or n, args.cpu_steps)
    if rank == 0 and world == 1 and not args.no_patterns:
        line["batched"] = bench_batched(torch)
        line["serving"] = bench_serving(torch, args.serve_requests)
        line["precision"] = bench_precision(torch)
    line["summary"] = summary(line)  # last key: the end of the printed line
    return line


def summary(line):
    """The headline numbers of every block, compact, for the end of the JSON line."""
    out = {"f64": {"cell_updates_per_s": line["value"], "e2e": round(line["e2e"]["value"], 1),
                   "stage_ms": line["roofline"]["stage_ms"], "frac_of_probe": line["roofline"]["frac"],
                   "frac_of_nominal": (line["roofline"].get("fp64_nominal") or {}).get("frac")}}
    if "fp32" in line:
        r = line["fp32"]["roofline"]
        out["f32"] = {"cell_updates_per_s": line["fp32"]["value"], "e2e": round(line["fp32"]["e2e"]["value"], 1),
                      "stage_ms": r["stage_ms"], "hbm_frac": r["hbm"]["frac"]}
    cpu = line.get("cpu_baseline")
    if cpu:
        out["cpu_baseline"] = {"cell_updates_per_s": round(cpu["value"], 1), "cores": cpu["cores"],
                               "f64_e2e_over_cpu": round(line["e2e"]["value"] / cpu["value"], 1)}
    b = line.get("batched")
    if b:
        out["batched"] = {k: b[k] for k in ("speedup", "batched_fp32_solves_per_s", "serial_fp64_solves_per_s",
                                             "max_l1_density_err_fp32_vs_fp64", "min_cycles_1024", "tile")}
    sv = line.get("serving")
    if sv:
        out["serving"] = {k: [v["solves_per_s"], v["speedup_vs_serial_fp64"], v["tts_p50_s"], v["tts_p99_s"],
                              v["arrival_bound"]]
                          for k, v in sv.items() if isinstance(v, dict) and "solves_per_s" in v}
        out["serving_fields"] = ["solves_per_s", "speedup_vs_serial_fp64", "p50_s", "p99_s", "arrival_bound"]
        for suffix, guarded in (("", True), ("_unguarded", False)):
            errs = [v["fp32_l1_density_err_vs_fp64_max"] for k, v in sv.items()
                    if isinstance(v, dict) and v.get("fp32_l1_density_err_vs_fp64_max") is not None
                    and ("unguarded" not in k) == guarded]
            out["serving_fp32_l1_max" + suffix] = max(errs) if errs else None
    p = line.get("precision")
    if p:
        out["precision_l1_density"] = {k: v["l1_density"] for k, v in p.items()}
    return out


# ---------------------------------------------------------------------------
# The three added patterns, each against the plain float64 path.
# ---------------------------------------------------------------------------
def ensemble_specs():
    """64 solves: 16 each of 128^2..1024^2, alternating KH (4 vars) and driven turbulence (3 vars)."""
    specs = []
    seed = 1
    for side in (128, 256, 512, 1024):
        for i in range(16):
            if i % 2 == 0:
                specs.append(("kh", side, None))
            else:
                specs.append(("turbulence", side, seed))
                seed += 1
    return specs


def make_request(kind, side, seed, tlim, dtype, rid=0):
    from jathenax_gb300.serve import Request
    return Request(rid=rid, arrival=0.0, problem=kind, side=side, reconstruct="ppm4", rsolver="roe",
                   tlim=tlim, dtype=dtype, seed=seed or 1)


def bench_batched(torch, tlim=0.05):
    """Batched ensemble (float32, one persistent launch per stage, graph-captured)
    against looping the plain float64 kernel over the same 64 solves."""
    from jathenax_gb300 import autotune
    from jathenax_gb300.batch import Batch, ClockBank
    from jathenax_gb300.diagnostics import relative_l1
    from jathenax_gb300.serve import build_solve
    reqs = [make_request(k, n, s, tlim, "float32", i) for i, (k, n, s) in enumerate(ensemble_specs())]
    tuned = autotune.tune_batch([build_solve(r, (0, 0)) for r in reqs])
    bank = ClockBank(len(reqs))
    solves = [build_solve(r, tuned["tile"], clock=bank.slot(i)) for i, r in enumerate(reqs)]
    batch = Batch(solves, blocks_per_sm=tuned["blocks_per_sm"], clocks=bank)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.run(steps_per_sync=16)
    torch.cuda.synchronize()
    batched_s = time.perf_counter() - t0
    out32 = [s.S.cpu().numpy() for s in solves]
    cycles = [c.cycle for c in bank.read()]
    del batch, solves
    t0 = time.perf_counter()
    l1 = []
    for r, u32 in zip(reqs, out32):
        s64 = build_solve(r, dtype="float64")
        s64.run(steps_per_sync=32)
        l1.append(float(relative_l1(u32, s64.S.cpu().numpy())[0]))
        del s64
    torch.cuda.synchronize()
    serial_s = time.perf_counter() - t0
    return {"solves": len(reqs), "workload": "16 each of 128^2/256^2/512^2/1024^2, KH (4 vars) and "
            f"driven turbulence (3 vars, seeds 1..32), ppm4+roe rk3, tlim {tlim}",
            "batched_fp32_solves_per_s": round(len(reqs) / batched_s, 3),
            "serial_fp64_solves_per_s": round(len(reqs) / serial_s, 3),
            "speedup": round(serial_s / batched_s, 2),
            "max_l1_density_err_fp32_vs_fp64": max(l1),
            "min_cycles_1024": min(c for c, r in zip(cycles, reqs) if r.side == 1024),
            "cycles_range": [min(cycles), max(cycles)],
            "tile": tuned["tile"], "blocks_per_sm": tuned["blocks_per_sm"],
            "autotune": {"chosen": tuned["knobs"], "ms_per_step": round(tuned["ms_per_step"], 4),
                         "knobs": ["staging", "columns_per_lane", "rows", "blocks_per_sm"],
                         "timing": tuned["timing"], "clock_mhz": tuned["clock_mhz"],
                         "trials": [[t["staging"], t["columns_per_lane"], t["rows"], t["blocks_per_sm"],
                                     round(t["ms_per_step"], 4)] for t in tuned["trials"]]},
            "batched_s": round(batched_s, 3), "serial_s": round(serial_s, 3)}


def bench_serving(torch, n):
    """Scaled serving stream: Poisson arrivals, side log-uniform 64..512, tlim U[0.02, 0.2],
    80% float32; continuous batching vs serial plain float64, at a light and a heavy rate
    (the same requests; only the arrival times differ)."""
    from jathenax_gb300.diagnostics import relative_l1
    from jathenax_gb300.serve import Server, make_stream, run_serial, warmup_requests

    def stream(rate):
        return make_stream(n, rate=rate, seed=2026, side_range=(64, 512), tlim_range=(0.02, 0.2))

    ref = stream(200.0)
    # Like each server below, the serial baseline first runs one tiny request
    # per method untimed, so CUDA's lazy kernel loading is charged to neither.
    run_serial(warmup_requests(("float64",)), dtype="float64")
    serial = run_serial(ref, dtype="float64", keep_results=True)
    out = {"requests": n, "stream": "Poisson arrivals, side log-uniform 64..512, tlim U[0.02,0.2], problems "
           "smooth/kh/turbulence, random recon/rsolver, 150 GB budget",
           "serial_fp64_solves_per_s": round(serial["solves_per_s"], 3),
           "warm": "one untimed pass of the stream first (device and pinned-host caching allocators, kernels)"}
    # One untimed pass of the same stream, so that no timed server pays for
    # first-time device and pinned-host allocations of its result sizes.
    warm = Server(budget_bytes=150e9, steps_per_tick=8, keep_results=True)
    warm.warmup()
    warm.run(stream(1000.0))
    del warm
    for rate in (200.0, 1000.0):
        for label, dtype, guard in (("mixed_80pct_fp32", None, True), ("all_fp32", "float32", True),
                                    ("all_fp32_unguarded", "float32", False)):
            reqs = stream(rate)
            server = Server(budget_bytes=150e9, steps_per_tick=8, keep_results=True, dtype=dtype, guard=guard)
            server.warmup()
            stats = server.run(reqs)
            errs = [float(relative_l1(q.result, r.result)[0]) for r, q in zip(ref, reqs)
                    if q.served_dtype == "float32"]
            # Requests offered per second over the arrival window: a server
            # whose solves/s comes within 20 % of it is bounded by the
            # arrivals, not by its own speed.
            window = max(q.arrival for q in reqs) - min(q.arrival for q in reqs)
            offered = (len(reqs) - 1) / window if window > 0 else float("inf")
            out[f"{label}_rate{int(rate)}"] = {
                "offered_per_s": round(offered, 1),
                "arrival_bound": bool(stats["solves_per_s"] >= 0.8 * offered),
                "solves_per_s": round(stats["solves_per_s"], 3),
                "speedup_vs_serial_fp64": round(stats["solves_per_s"] / serial["solves_per_s"], 2),
                "tts_p50_s": round(stats["tts_p50_s"], 4), "tts_p99_s": round(stats["tts_p99_s"], 4),
                "peak_live": stats["peak_live"], "promoted_to_float64": stats["promoted_to_float64"],
                "fp32_l1_density_err_vs_fp64_max": max(errs) if errs else None,
                "fp32_l1_density_err_vs_fp64_median": float(np.median(errs)) if errs else None}
    out["tiles"] = server.tile_table()
    return out


def bench_serving_stated(args):
    """The serving stream as stated: Poisson arrivals, grid side log-uniform in
    64..2048, problem uniform over smooth/KH/turbulence, random reconstruction and
    Riemann solver, tlim uniform in [0.2, 3], 80 % float32, 150 GB budget; the
    first --serve-stated requests of the seeded stream. Serial float64 on the same
    requests is the baseline and the float64 rerun of every float32 result."""
    import torch
    from jathenax_gb300.diagnostics import relative_l1
    from jathenax_gb300.serve import Server, make_stream, run_serial, warmup_requests
    torch.cuda.set_device(0)
    n, rate = args.serve_stated, args.serve_rate

    def stream():
        return make_stream(n, rate=rate, seed=2026, side_range=(64, 2048), tlim_range=(0.2, 3.0))

    ref = stream()
    run_serial(warmup_requests(("float64",)), dtype="float64")
    serial = run_serial(ref, dtype="float64", keep_results=True)
    out = {"requests": n, "rate": rate, "stream": "Poisson arrivals, side log-uniform 64..2048, tlim U[0.2,3], "
           "problems smooth/kh/turbulence, random recon/rsolver, 80% float32, 150 GB budget, seed 2026",
           "sides": [min(r.side for r in ref), int(np.median([r.side for r in ref])), max(r.side for r in ref)],
           "cell_updates": int(sum(r.side ** 2 * r.cycles for r in ref)),
           "serial_fp64_s": round(serial["elapsed_s"], 2), "serial_fp64_solves_per_s": round(serial["solves_per_s"], 4)}
    for label, dtype in (("mixed_80pct_fp32", None), ("all_fp32_unguarded", "float32")):
        reqs = stream()
        server = Server(budget_bytes=150e9, steps_per_tick=8, keep_results=True, dtype=dtype,
                        guard=dtype is None)
        server.warmup()
        stats = server.run(reqs)
        errs = [float(relative_l1(q.result, r.result)[0]) for r, q in zip(ref, reqs) if q.served_dtype == "float32"]
        window = max(q.arrival for q in reqs) - min(q.arrival for q in reqs)
        offered = (len(reqs) - 1) / window if window > 0 else float("inf")
        out[label] = {"solves_per_s": round(stats["solves_per_s"], 4), "elapsed_s": round(stats["elapsed_s"], 2),
                      "speedup_vs_serial_fp64": round(stats["solves_per_s"] / serial["solves_per_s"], 2),
                      "tts_p50_s": round(stats["tts_p50_s"], 3), "tts_p99_s": round(stats["tts_p99_s"], 3),
                      "offered_per_s": round(offered, 2), "arrival_bound": bool(stats["solves_per_s"] >= 0.8 * offered),
                      "peak_live": stats["peak_live"], "peak_gb": round(stats["peak_bytes"] / 1e9, 1),
                      "failed": stats["failed"], "promoted_to_float64": stats["promoted_to_float64"],
                      "fp32_requests": len(errs),
                      "fp32_l1_density_err_vs_fp64_max": max(errs) if errs else None,
                      "fp32_l1_density_err_vs_fp64_median": float(np.median(errs)) if errs else None,
                      "fp32_over_1e-5": sum(e > 1e-5 for e in errs)}
        out[f"{label}_tiles"] = server.tile_table()
        del server
    print(json.dumps(out), flush=True)


def driven_turbulence(side, tlim, dtype, smagorinsky_cs=0.0, seed=1618):
    """The reference's driven-turbulence run (input.py:43-47 forcing, run.py:133-158):
    rest state, 56 parabolic modes (3 <= |k| <= 5), seed 1618, nu 1.5e-6, drag 0.3333335."""
    import torch
    from jathenax_gb300.forcing import cartesian_modes, forcing_basis, modal_coefficients
    from jathenax_gb300.initial_conditions import cell_centers, uniform_rest
    from jathenax_gb300.solver import Solve
    x, _ = cell_centers(side, side)
    modes = cartesian_modes(3, 5, (-5, 5), (-5, 5))
    updates = int(np.ceil(tlim / 0.0075)) + 1
    table = modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, seed, 0.75, 0.0075, updates)
    basis = forcing_basis(modes, x, x, (1.0, 1.0))
    return Solve(uniform_rest(side, side), 1 / side, 1 / side, 1.0, 1.17549e-38, "rk3", 0.4, tlim, 10**8,
                 viscosity=1.5e-6, smagorinsky_cs=smagorinsky_cs, drag_rate=0.3333335,
                 forcing=(table, basis), dt_update=0.0075, dedt=0.03703705, dtype=getattr(torch, dtype))


def bench_precision(torch):
    """FP32 state against the FP64 run of the same problem at the same end time."""
    from jathenax_gb300.diagnostics import precision_report
    from jathenax_gb300.serve import build_solve
    out = {}
    runs = [("kh_512_t0.05", lambda dt: build_solve(make_request("kh", 512, 1618, 0.05, dt), dtype=dt)),
            ("turbulence_256_t0.1",
             lambda dt: build_solve(make_request("turbulence", 256, 1618, 0.1, dt), dtype=dt)),
            ("turbulence_1024_t1", lambda dt: driven_turbulence(1024, 1.0, dt)),
            ("turbulence_smagorinsky0.17_1024_t1", lambda dt: driven_turbulence(1024, 1.0, dt, 0.17))]
    for name, make in runs:
        res, cycles, seconds = {}, {}, {}
        for dtype in ("float32", "float64"):
            s = make(dtype)
            U0 = s.S.cpu().numpy().astype(np.float64)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run(steps_per_sync=64)
            torch.cuda.synchronize()
            seconds[dtype] = round(time.perf_counter() - t0, 3)
            res[dtype] = s.S.cpu().numpy()
            cycles[dtype] = s.state().cycle
            del s
        side = res["float64"].shape[0]
        out[name] = precision_report(res["float32"], res["float64"], U0, 1 / side, 1 / side)
        out[name].update(cycles=cycles, seconds=seconds)
    return out


def bench_ensemble(args):
    """Batched cycles of the 64-solve ensemble (or one half) at one tile: one JSON line."""
    import torch
    from jathenax_gb300.batch import Batch
    from jathenax_gb300.serve import build_solve
    torch.cuda.set_device(0)
    tile = tuple(int(v) for v in args.tile.lower().split("x"))
    reqs = [make_request(k, n, s, 1.0, "float32", i) for i, (k, n, s) in enumerate(ensemble_specs())
            if args.ensemble == "all" or k == args.ensemble]
    batch = Batch([build_solve(r, tile) for r in reqs])
    for _ in range(args.warmup):
        batch.enqueue_step()
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    start.record(stream)
    for _ in range(args.steps):
        batch.enqueue_step()
    end.record(stream)
    end.synchronize()
    cells = sum(r.side * r.side for r in reqs)
    ms = start.elapsed_time(end) / max(args.steps, 1)
    print(json.dumps({"workload": f"{len(reqs)} float32 solves ({args.ensemble}) of the 64-solve ensemble, "
                                  f"ppm4+roe rk3, tile {tile[0]}x{tile[1]}",
                      "cells": cells, "steps": args.steps, "warmup": args.warmup, "ms_per_cycle": round(ms, 4),
                      "cell_updates_per_s": round(cells / ms * 1e3, 1)}), flush=True)


def bench_turbulence_long(args):
    """The driven-turbulence configuration to a long end time in both precisions (one JSON line).

    With ``--average-from T0`` the KE shell spectrum is also averaged over the
    snapshots at T0, T0 + 1, ..., tlim (each run stops exactly at those times)
    and compared as time averages. With ``--chaos-floor`` a third, float64 run
    starts from the same state with the density perturbed by 1e-12 (relative,
    seeded noise): its distance from the float64 run is the chaotic
    divergence that no precision can remove, the scale the float32 numbers are
    read against.
    """
    import torch
    from jathenax_gb300.diagnostics import precision_report, shell_spectra
    torch.cuda.set_device(0)
    side = args.n or 1024
    tlim = args.turbulence_t
    samples = [] if args.average_from is None else \
        [float(t) for t in np.arange(args.average_from, tlim + 0.5, 1.0) if t <= tlim]
    runs = [("float32", "float32", 0.0), ("float64", "float64", 0.0)]
    if args.chaos_floor:
        runs.append(("float64_perturbed", "float64", 1e-12))
    res, info, spectra = {}, {}, {}
    U0 = None
    for name, dtype, eps in runs:
        s = driven_turbulence(side, tlim, dtype, smagorinsky_cs=args.cs)
        if U0 is None:
            U0 = s.S.cpu().numpy().astype(np.float64)
        if eps:
            noise = np.random.default_rng(45).standard_normal(U0.shape[:2])
            s.S[..., 0] *= torch.as_tensor(1.0 + eps * noise, device=s.S.device, dtype=s.S.dtype)
        acc = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for stop in samples + [tlim]:
            s.set_clock(tlim=stop, done=0)
            s.run(steps_per_sync=256)
            if stop in samples:
                acc.append(shell_spectra(s.S.cpu().numpy())[1])
        torch.cuda.synchronize()
        seconds = time.perf_counter() - t0
        state = s.state()
        res[name] = s.S.cpu().numpy()
        if acc:
            spectra[name] = np.mean(acc, axis=0)
        info[name] = {"cycles": state.cycle, "time": state.time, "seconds": round(seconds, 2),
                      "cell_updates_per_s": round(side * side * state.cycle / seconds, 1)}
        del s

    def mean_spectrum_dev(a, b, kmax):
        sl = slice(1, kmax)
        return float(np.max(np.abs(spectra[a][sl] - spectra[b][sl]) / np.maximum(spectra[b][sl], 1e-300)))

    out = {"workload": f"driven turbulence {side}^2, rk3 ppm4 roe, seed 1618, nu 1.5e-6, drag 0.3333335, "
                       f"Cs {args.cs}, t={tlim}",
           "precision": precision_report(res["float32"], res["float64"], U0, 1 / side, 1 / side), "runs": info}
    if args.chaos_floor:
        out["chaos_floor"] = precision_report(res["float64_perturbed"], res["float64"], U0, 1 / side, 1 / side)
    if spectra:
        out["time_averaged_spectrum"] = {"times": samples}
        for name in spectra:
            if name == "float64":
                continue
            out["time_averaged_spectrum"][f"{name}_vs_float64"] = {
                f"max_rel_dev_k<{k}": mean_spectrum_dev(name, "float64", k) for k in (16, 64, side // 2)}
    print(json.dumps(out), flush=True)


def bench_reference(args, world, rank):
    """The reference algorithm's CPU path (the float64 oracle port) on host cores."""
    if rank != 0:
        return None
    n = args.cpu_sample or args.n or 4096
    base = cpu_baseline_sample(n, max(1, min(args.steps, 8)))
    seconds = base.pop("seconds")
    return {
        "impl": "reference", "metric": METRIC, "value": round(base["value"], 1), "unit": METRIC,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, world),
        "cpu_baseline": dict(base),
        "e2e": {"value": round(base["value"], 1), "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "seconds": seconds,
    }


def bench_precision_sweep(args):
    """Float32 vs float64 L1 density error per (problem, method, side, end time) as served
    (the serving set-ups, build_solve), one JSON line each: the evidence behind serve.py's
    float32 precision guard (serve.FP32_ERR)."""
    import torch
    from jathenax_gb300.diagnostics import relative_l1
    from jathenax_gb300.serve import PROBLEMS, RECONS, SOLVERS, Request, build_solve
    torch.cuda.set_device(0)
    sides = (64, 85, 128, 256) if args.n is None else (args.n,)
    tlims = tuple(float(t) for t in args.precision_tlims.split(","))
    pairs = None if not args.precision_pairs else {tuple(p.split(":")) for p in args.precision_pairs.split(",")}
    for problem in PROBLEMS:
        for recon in RECONS:
            if pairs is not None and (problem, recon) not in pairs:
                continue
            for rsolver in SOLVERS:
                for side in sides:
                    # One run per precision, stopped at each end time in turn (the first
                    # stop is exactly a request with that end time; each later one
                    # includes the earlier stops' clipped steps, in both precisions alike).
                    req = Request(rid=0, arrival=0.0, problem=problem, side=side, reconstruct=recon,
                                  rsolver=rsolver, tlim=max(tlims), dtype="float32", seed=7)
                    solves = {dtype: build_solve(req, dtype=dtype) for dtype in ("float32", "float64")}
                    for tlim in sorted(tlims):
                        out = {}
                        for dtype, s in solves.items():
                            s.set_clock(tlim=tlim, done=0)
                            s.run(steps_per_sync=64)
                            out[dtype] = (s.S.cpu().numpy(), s.state())
                        l1 = relative_l1(out["float32"][0], out["float64"][0])
                        print(json.dumps({"problem": problem, "method": f"{recon}/{rsolver}", "side": side,
                                          "tlim": tlim, "l1_density": float(l1[0]), "l1_max": float(np.max(l1)),
                                          "cycles": [out["float32"][1].cycle, out["float64"][1].cycle]}),
                              flush=True)
                    del solves


def bench_sweep(args):
    """cell-updates/s of every method combination (graph replays of whole cycles)."""
    import torch
    from jathenax_gb300 import _lib
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    from jathenax_gb300.solver import Solve
    n = args.n or 1024
    U0 = torch.as_tensor(kelvin_helmholtz_tanh(n, n), device="cuda")
    for dtype in (torch.float64, torch.float32):
        for recon in ("dc", "plm", "ppm4", "ppmx", "wenoz"):
            for rsolver in ("llf", "hlle", "roe"):
                for integrator in ("rk2", "rk3", "rk4"):
                    s = Solve(U0, 1.0 / n, 1.0 / n, 1.0, 1e-10, integrator, 0.4, 1e30, 2**31 - 1,
                              reconstruct=recon, rsolver=rsolver, dtype=dtype)
                    s.capture(1)
                    for _ in range(args.warmup):
                        s.graph.replay()
                    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    torch.cuda.synchronize()
                    start.record()
                    for _ in range(args.steps):
                        s.graph.replay()
                    end.record()
                    torch.cuda.synchronize()
                    ms = start.elapsed_time(end) / args.steps
                    tx, ty, smem = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
                    _lib.call("jx_tile_info", ctypes.byref(s.desc), ctypes.byref(tx), ctypes.byref(ty),
                              ctypes.byref(smem))
                    print(json.dumps({"sweep": f"{recon}/{rsolver}/{integrator}", "dtype": str(dtype)[6:],
                                      "n": n, "ms_per_step": round(ms, 4),
                                      "value": round(n * n / (ms * 1e-3), 1), "unit": METRIC,
                                      "tile": [tx.value, ty.value]}), flush=True)
                    del s


def main():
    args = parse_args()
    if args.sweep:
        bench_sweep(args)
        return
    if args.precision_sweep:
        bench_precision_sweep(args)
        return
    if args.serve_stated:
        bench_serving_stated(args)
        return
    if args.turbulence_t is not None:
        bench_turbulence_long(args)
        return
    if args.ensemble is not None:
        bench_ensemble(args)
        return
    args.n = args.n or 4096
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        line = bench_reference(args, world, rank)
    else:
        line = bench_ours(args, world, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
