"""Autotuner for the stage kernels of a batch (and of the serving loop).

Knobs, every one reported with each trial and the choice:

* ``staging``: how a tile's halo reaches the stencil. ``"shared"`` stages a
  32 x h tile plus its halo in shared memory (256 threads, one cell or more
  per thread); ``"march"`` keeps a 5-row window in registers while one warp
  walks the tile down its rows (no shared memory, no barriers).
* ``columns_per_lane`` (marching only): 1, 2 or 3 columns of cells per
  thread, i.e. tiles 26, 58 or 90 columns wide (6 of the 32 x columns are the
  two 3-cell halos). More columns spread the halo over more outputs and give
  each thread more independent work; fewer leave more warps per grid and
  fewer registers per thread.
* ``rows``: the tile height h (cells per thread along y for the marching
  walk, 8 h / 256 cells per thread for the shared-memory tile).
* ``blocks_per_sm``: resident persistent blocks per SM of the batched stage
  kernels (0: as many as occupancy allows).

Float32 results do not depend on any knob (every rounding is explicit);
float64 results agree across knobs to rounding (marching and shared-memory
kernels contract different products). Float64 marches with two columns per
lane only.

Each candidate starts from the same states and clocks (restored before it
runs, so a solve that reaches its end time during the search does so in
every candidate alike), runs ``warmup`` untimed and ``repeats`` x ``steps``
timed batched cycles (CUDA events); its time is the median repeat, and the
SM clock (``nvidia-smi``) is read before and after the search. Probe-grid
results (:func:`tune`) are cached per GPU model in memory and in
``$JATHENAX_GB300_CACHE`` (default ``~/.cache/jathenax_gb300/autotune.json``).
"""

import json
import os
import shutil
import statistics
import subprocess
from pathlib import Path

from . import _lib

SHARED_TILES = ((32, 8), (32, 16), (32, 32))
MARCH_TILES = tuple((w, h) for w in (26, 58, 90) for h in (8, 16, 32))
BLOCKS_PER_SM = (0, 1, 2)
_memory = {}


def tiles_for(dtype):
    """Candidate tiles of a precision (float64 marches with 58-column tiles only)."""
    march = MARCH_TILES if dtype == "float32" else tuple(t for t in MARCH_TILES if t[0] == 58)
    return SHARED_TILES + march


def knobs(tile, blocks_per_sm):
    """The knob values of one candidate."""
    march = tile[0] in (26, 58, 90)
    return {"staging": "march" if march else "shared",
            "columns_per_lane": (tile[0] + 6) // 32 if march else None,
            "tile": list(tile), "rows": tile[1], "blocks_per_sm": blocks_per_sm}


def sm_clock_mhz():
    """Current SM clock of the visible GPU from nvidia-smi (None where it is not available)."""
    if shutil.which("nvidia-smi") is None:
        return None
    index = (os.environ.get("CUDA_VISIBLE_DEVICES") or "0").split(",")[0].strip() or "0"
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.sm", "--format=csv,noheader,nounits", "-i", index],
                             capture_output=True, text=True, timeout=10)
        return float(out.stdout.strip().splitlines()[0])
    except (OSError, ValueError, IndexError, subprocess.SubprocessError):
        return None


def time_batch(batch, steps, repeats, warmup):
    """Milliseconds per batched cycle of each of `repeats` runs of `steps` cycles."""
    t = _lib.torch()
    for _ in range(warmup):
        batch.enqueue_step()
    start, end = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    out = []
    for _ in range(repeats):
        start.record()
        for _ in range(steps):
            batch.enqueue_step()
        end.record()
        end.synchronize()
        out.append(start.elapsed_time(end) / steps)
    return out


def tune_batch(solves, tiles=None, blocks_per_sm=BLOCKS_PER_SM, steps=10, repeats=2, warmup=2):
    """Pick the knobs for one particular set of solves by timing the batched
    cycle itself. The solves are retiled in place (Solve.set_tile); their
    states and clocks are put back before every candidate and at the end, but
    forcing caches and CFL partials are not, so build fresh ones for the real
    run.

    Returns {"knobs", "tile", "blocks_per_sm", "ms_per_step", "trials",
    "clock_mhz", "timing"} (not cached: the answer belongs to the solve set).
    """
    from .batch import Batch
    dtypes = {str(s.S.dtype).replace("torch.", "") for s in solves}
    if tiles is None:
        tiles = tiles_for("float32" if dtypes == {"float32"} else "float64")
    clock_before = sm_clock_mhz()
    saved = [(s.S.clone(), s.clock.clone()) for s in solves]

    def restore():
        for s, (state, clock) in zip(solves, saved):
            s.S.copy_(state)
            s.clock.copy_(clock)

    trials = []
    for tile in tiles:
        restore()
        try:
            for s in solves:
                s.set_tile(tile)
        except (ValueError, RuntimeError):  # e.g. the tile does not fit in shared memory
            continue
        for bps in blocks_per_sm:
            restore()
            runs = time_batch(Batch(solves, blocks_per_sm=bps), steps, repeats, warmup)
            trials.append(dict(knobs(tile, bps), ms_per_step=statistics.median(runs),
                               repeats_ms=[round(r, 4) for r in runs]))
    restore()
    if not trials:
        raise RuntimeError("no autotuning candidate could run")
    best = min(trials, key=lambda r: r["ms_per_step"])
    return {"knobs": {k: best[k] for k in ("staging", "columns_per_lane", "rows", "blocks_per_sm")},
            "tile": best["tile"], "blocks_per_sm": best["blocks_per_sm"], "ms_per_step": best["ms_per_step"],
            "trials": trials, "clock_mhz": [clock_before, sm_clock_mhz()],
            "timing": f"{warmup} warm-up + {repeats} x {steps} timed batched cycles per candidate, median repeat"}


def _cache_path():
    root = os.environ.get("JATHENAX_GB300_CACHE")
    return Path(root) if root else Path.home() / ".cache" / "jathenax_gb300" / "autotune.json"


def _load():
    try:
        return json.loads(_cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(key, value):
    data = _load()
    data[key] = value
    try:
        path = _cache_path()
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(data, indent=1, sort_keys=True))
    except OSError:
        pass


def _probe_solves(dtype, reconstruct, rsolver, nvar, side, count):
    t = _lib.torch()
    from .initial_conditions import kelvin_helmholtz_tanh, smooth_waves
    from .solver import Solve
    U = kelvin_helmholtz_tanh(side, side) if nvar == 4 else smooth_waves(side, side)
    return [Solve(U, 1.0 / side, 1.0 / side, 1.0, 1e-10, "rk3", 0.4, 1e30, 2**31 - 1, reconstruct=reconstruct,
                  rsolver=rsolver, dtype=getattr(t, dtype)) for _ in range(count)]


def tune(dtype="float32", reconstruct="ppm4", rsolver="roe", nvar=4, side=1024, count=1, steps=10, repeats=2,
         blocks_per_sm=(0,), use_cache=True):
    """Knobs for `count` probe solves of one kernel class on side x side grids
    (cached per GPU model). Returns the :func:`tune_batch` result."""
    t = _lib.torch()
    key = "|".join(map(str, ("v3", t.cuda.get_device_name(), dtype, reconstruct, rsolver, nvar, side, count)))
    if use_cache:
        if key in _memory:
            return _memory[key]
        stored = _load().get(key)
        if stored:
            _memory[key] = stored
            return stored
    result = tune_batch(_probe_solves(dtype, reconstruct, rsolver, nvar, side, count),
                        tiles=tiles_for(dtype), blocks_per_sm=blocks_per_sm, steps=steps, repeats=repeats)
    result["key"] = key
    _memory[key] = result
    _store(key, result)
    return result
