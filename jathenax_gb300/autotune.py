"""Autotuner for the batched stage kernels.

Searches the stage tile (the shared-memory kernel's 32 x 8, 16 or 32 tiles
of 256 threads, and the register-marching kernel's 58 x 8 / 16 / 32 tiles
of 128 threads) and the number of persistent blocks per SM (occupancy limit
or 1..4) for one (precision, reconstruction, Riemann solver, variable count)
kernel class on a probe grid, timing a few evolve cycles of each candidate
with CUDA events. Within one kernel the tile never changes results (each
cell's arithmetic is the same and the CFL reduction is an exact maximum);
the two kernels agree to rounding. Choices are cached per GPU model in
memory and in ``$JATHENAX_GB300_CACHE`` (default
``~/.cache/jathenax_gb300/autotune.json``).
"""

import json
import os
from pathlib import Path

from . import _lib

TILES = ((32, 8), (32, 16), (32, 32), (58, 8), (58, 16), (58, 32))
BLOCKS_PER_SM = (0, 1, 2, 3, 4)
_memory = {}


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


def _probe_state(nvar, side):
    from .initial_conditions import kelvin_helmholtz_tanh, smooth_waves
    return kelvin_helmholtz_tanh(side, side) if nvar == 4 else smooth_waves(side, side)


def measure(dtype, reconstruct, rsolver, nvar, side, tile, blocks_per_sm, steps=4):
    """Milliseconds per evolve cycle of one probe solve run through the batch path."""
    t = _lib.torch()
    from .batch import Batch
    from .solver import Solve
    solve = Solve(_probe_state(nvar, side), 1.0 / side, 1.0 / side, 1.0, 1e-10, "rk3", 0.4, 1e30,
                  2**31 - 1, reconstruct=reconstruct, rsolver=rsolver, tile=tuple(tile),
                  dtype=getattr(t, dtype))
    batch = Batch([solve], blocks_per_sm=blocks_per_sm)
    for _ in range(2):
        batch.enqueue_step()
    start, end = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        batch.enqueue_step()
    end.record()
    end.synchronize()
    return start.elapsed_time(end) / steps


def tune(dtype="float32", reconstruct="ppm4", rsolver="roe", nvar=4, side=1024, steps=4,
         use_cache=True):
    """Return {"tile": [tx, ty], "blocks_per_sm": ..., "ms_per_step": ..., "trials": [...]}."""
    t = _lib.torch()
    key = "|".join(map(str, ("v2", t.cuda.get_device_name(), dtype, reconstruct, rsolver, nvar, side)))
    if use_cache:
        if key in _memory:
            return _memory[key]
        stored = _load().get(key)
        if stored:
            _memory[key] = stored
            return stored
    trials = []
    for tile in TILES:
        for bps in BLOCKS_PER_SM:
            try:
                ms = measure(dtype, reconstruct, rsolver, nvar, side, tile, bps, steps)
            except (ValueError, RuntimeError):  # tile does not fit in shared memory
                continue
            trials.append({"tile": list(tile), "blocks_per_sm": bps, "ms_per_step": ms})
    if not trials:
        raise RuntimeError("no autotuning candidate could run")
    best = min(trials, key=lambda r: r["ms_per_step"])
    result = dict(best, trials=trials, key=key)
    _memory[key] = result
    _store(key, result)
    return result


def tune_batch(make_solves, tiles=TILES, blocks_per_sm=(0,), steps=3, warmup=2):
    """Pick the tile (and persistent blocks per SM) for one particular set of
    solves, timing the batched cycle itself rather than a probe grid.

    ``make_solves(tile)`` returns fresh Solve objects built with that tile;
    each candidate runs ``warmup`` untimed and ``steps`` timed batched cycles.
    Returns {"tile", "blocks_per_sm", "ms_per_step", "trials"} (not cached:
    the answer belongs to the solve set).
    """
    t = _lib.torch()
    from .batch import Batch
    trials = []
    for tile in tiles:
        for bps in blocks_per_sm:
            try:
                solves = make_solves(tuple(tile))
            except (ValueError, RuntimeError):  # tile does not fit in shared memory
                continue
            batch = Batch(solves, blocks_per_sm=bps)
            for _ in range(warmup):
                batch.enqueue_step()
            start, end = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            start.record()
            for _ in range(steps):
                batch.enqueue_step()
            end.record()
            end.synchronize()
            trials.append({"tile": list(tile), "blocks_per_sm": bps, "ms_per_step": start.elapsed_time(end) / steps})
            del batch, solves
    if not trials:
        raise RuntimeError("no autotuning candidate could run")
    best = min(trials, key=lambda r: r["ms_per_step"])
    return dict(best, trials=trials)
