"""Serving: a continuously batched request loop over device-resident solves.

Requests (problem, grid side, reconstruction, Riemann solver, end time,
precision, seed) arrive over time. A request is admitted when it has arrived
and its device memory (three states, workspace, forcing tables) fits in the
HBM budget next to the live solves; it then stays resident on the GPU until
it reaches its end time. Every tick advances all live solves together through
one :class:`jathenax_gb300.batch.Batch` step per cycle; between ticks
finished solves leave (their memory returns to the budget) and waiting
requests join, so new work overlaps with solves already on the device.
Because batches are exact (a solve's result does not depend on its
neighbours), each result equals the result of running that request alone.

The reported metrics are time-to-solution (completion minus arrival:
queueing + compute) percentiles and solves per second.
"""

import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib

PROBLEMS = ("smooth", "kh", "turbulence")
RECONS = ("dc", "plm", "ppm4", "ppmx", "wenoz")
SOLVERS = ("llf", "hlle", "roe")


@dataclass
class Request:
    rid: int
    arrival: float        # seconds after the stream starts
    problem: str
    side: int
    reconstruct: str
    rsolver: str
    tlim: float
    dtype: str            # "float32" or "float64"
    seed: int
    admitted: float = None
    finished: float = None
    cycles: int = 0
    error: str = None
    served_dtype: str = None  # the precision the server ran it in (see served_dtype)
    result: object = field(default=None, repr=False)


def make_stream(n, rate, seed=0, side_range=(64, 2048), tlim_range=(0.2, 3.0), fp32_fraction=0.8,
                problems=PROBLEMS, recons=RECONS, solvers=SOLVERS):
    """Poisson arrivals at `rate` per second; side log-uniform; tlim uniform."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    lo, hi = np.log(side_range[0]), np.log(side_range[1])
    out = []
    for i in range(n):
        side = int(round(float(np.exp(rng.uniform(lo, hi)))))
        out.append(Request(
            rid=i, arrival=float(arrivals[i]), problem=str(rng.choice(problems)), side=max(side, 6),
            reconstruct=str(rng.choice(recons)), rsolver=str(rng.choice(solvers)),
            tlim=float(rng.uniform(*tlim_range)),
            dtype="float32" if rng.random() < fp32_fraction else "float64",
            seed=int(rng.integers(1, 2**31 - 1))))
    return out


# Stage tile of a request built without a tile choice (build_solve's
# default): the 32 x 16 shared-memory tile in both precisions.
SERVING_TILES = {"float32": (32, 16), "float64": (32, 16)}

# Size classes of served grids, for the tuned tiles: (largest side of the
# class, side of its probe grids, probe solves). The bounds split the served
# 64..2048 range into three geometric thirds.
SIZE_CLASSES = ((203, 114, 8), (645, 362, 4), (1 << 30, 1149, 2))


def size_class(side):
    return next(i for i, (top, _, _) in enumerate(SIZE_CLASSES) if side <= top)


# Float32 precision guard. FP32_ERR holds, per (problem, reconstruction),
# the worst float32-vs-float64 L1 density error measured over the three
# Riemann solvers, one row per side of FP32_ERR_SIDES and one column per end
# time of FP32_ERR_TLIMS (GB300: `bench.py --precision-sweep` with
# `--precision-tlims 0.1,0.2` and the default 0.5..3, each also with
# `--n 512`; values rounded up to two digits). Two mechanisms make it grow,
# both properties of the flows and limiters rather than of float32
# arithmetic as such: the shear layers (and, later, the waves) are chaotic,
# so any rounding difference grows - a float64 run perturbed in its 15th
# digit drifts from the unperturbed one by the same factors; and PPMX's
# smooth-extremum limiter takes discrete branches (curvature signs, the
# 1e-12 relative threshold, the extremum test on exactly equal neighbours)
# that these symmetric set-ups put on exact ties, which rounding moves -
# most on the under-resolved shear layers of sides 64 and 85.
FP32_ERR_SIDES = (64, 85, 128, 256, 512)
FP32_ERR_TLIMS = (0.1, 0.2, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0)
FP32_ERR = {
    ("kh", "dc"): (
        (7.8e-08, 7.3e-08, 8.6e-08, 7.0e-08, 9.9e-08, 3.4e-07, 5.2e-07, 7.8e-07),  # 64
        (6.9e-08, 6.9e-08, 8.1e-08, 8.9e-08, 1.5e-07, 4.0e-07, 7.9e-07, 9.8e-07),  # 85
        (9.2e-08, 9.0e-08, 8.8e-08, 1.2e-07, 1.6e-07, 4.5e-07, 9.1e-07, 1.6e-06),  # 128
        (1.5e-07, 1.6e-07, 1.3e-07, 1.8e-07, 3.8e-07, 8.8e-07, 1.6e-06, 2.5e-06),  # 256
        (3.5e-07, 4.0e-07, 3.9e-07, 6.2e-07, 1.4e-06, 2.0e-06, 3.4e-06, 8.7e-06),  # 512
    ),
    ("kh", "plm"): (
        (1.3e-07, 1.4e-07, 1.3e-07, 1.6e-07, 2.4e-07, 5.5e-07, 2.0e-06, 8.4e-06),  # 64
        (1.3e-07, 1.4e-07, 1.4e-07, 2.3e-07, 4.4e-07, 8.3e-07, 7.1e-07, 1.1e-06),  # 85
        (1.4e-07, 1.6e-07, 1.7e-07, 5.4e-07, 1.5e-06, 2.3e-06, 8.7e-06, 3.7e-05),  # 128
        (2.1e-07, 2.4e-07, 2.9e-07, 1.7e-06, 7.5e-06, 2.2e-05, 8.8e-05, 3.3e-04),  # 256
        (4.1e-07, 5.2e-07, 7.5e-07, 1.4e-06, 4.9e-06, 1.5e-05, 8.0e-05, 2.9e-04),  # 512
    ),
    ("kh", "ppm4"): (
        (1.4e-07, 1.9e-07, 2.2e-07, 3.6e-07, 9.2e-07, 9.0e-07, 2.1e-06, 9.6e-06),  # 64
        (1.8e-07, 2.3e-07, 3.1e-07, 6.3e-07, 1.9e-06, 2.4e-06, 3.5e-06, 6.6e-06),  # 85
        (2.2e-07, 2.9e-07, 3.6e-07, 9.4e-07, 5.0e-06, 1.7e-05, 7.0e-05, 2.3e-04),  # 128
        (3.3e-07, 4.2e-07, 5.5e-07, 2.4e-06, 2.1e-05, 3.8e-05, 7.8e-05, 2.6e-04),  # 256
        (5.4e-07, 7.3e-07, 8.6e-07, 2.2e-06, 1.4e-05, 4.8e-05, 1.8e-04, 7.0e-04),  # 512
    ),
    ("kh", "ppmx"): (
        (3.0e-06, 2.1e-05, 7.9e-05, 1.9e-04, 6.5e-04, 2.0e-03, 6.0e-03, 2.0e-02),  # 64
        (7.0e-06, 4.3e-05, 2.3e-04, 1.3e-03, 5.9e-03, 9.1e-03, 1.3e-02, 1.5e-02),  # 85
        (4.3e-07, 1.2e-06, 2.5e-06, 3.3e-05, 1.5e-04, 2.2e-04, 4.1e-04, 9.9e-04),  # 128
        (3.6e-07, 6.1e-07, 1.9e-06, 1.3e-05, 7.9e-05, 2.1e-04, 5.3e-04, 1.7e-03),  # 256
        (5.7e-07, 7.8e-07, 1.1e-06, 4.1e-06, 7.0e-05, 3.4e-04, 7.6e-04, 1.4e-03),  # 512
    ),
    ("kh", "wenoz"): (
        (2.7e-07, 3.0e-07, 2.8e-07, 3.2e-07, 4.5e-07, 7.8e-07, 2.4e-06, 1.1e-05),  # 64
        (2.1e-07, 2.6e-07, 2.9e-07, 4.3e-07, 9.5e-07, 1.7e-06, 1.9e-06, 3.4e-06),  # 85
        (1.7e-07, 2.7e-07, 3.3e-07, 8.2e-07, 2.7e-06, 6.5e-06, 2.4e-05, 8.9e-05),  # 128
        (2.3e-07, 2.9e-07, 3.7e-07, 1.5e-06, 1.1e-05, 2.8e-05, 1.4e-04, 5.2e-04),  # 256
        (4.1e-07, 5.3e-07, 7.0e-07, 1.5e-06, 6.5e-06, 1.6e-05, 4.1e-05, 2.3e-04),  # 512
    ),
    ("smooth", "dc"): (
        (5.7e-08, 6.6e-08, 6.4e-08, 6.6e-08, 6.6e-08, 7.1e-08, 6.8e-08, 6.7e-08),  # 64
        (6.5e-08, 6.4e-08, 6.7e-08, 6.6e-08, 6.8e-08, 6.3e-08, 6.6e-08, 6.5e-08),  # 85
        (6.3e-08, 5.7e-08, 6.1e-08, 6.6e-08, 7.9e-08, 7.7e-08, 7.5e-08, 6.7e-08),  # 128
        (5.8e-08, 5.7e-08, 7.0e-08, 6.9e-08, 8.1e-08, 7.4e-08, 7.4e-08, 7.3e-08),  # 256
        (6.5e-08, 7.5e-08, 7.6e-08, 7.3e-08, 7.9e-08, 7.7e-08, 8.1e-08, 8.6e-08),  # 512
    ),
    ("smooth", "plm"): (
        (7.2e-08, 8.6e-08, 1.1e-07, 1.2e-07, 1.2e-07, 1.4e-07, 1.4e-07, 1.4e-07),  # 64
        (8.1e-08, 9.2e-08, 9.7e-08, 1.2e-07, 1.3e-07, 1.3e-07, 1.6e-07, 1.7e-07),  # 85
        (8.3e-08, 9.2e-08, 1.2e-07, 1.4e-07, 1.5e-07, 1.5e-07, 1.6e-07, 1.6e-07),  # 128
        (8.9e-08, 1.2e-07, 1.3e-07, 1.5e-07, 1.7e-07, 1.7e-07, 1.9e-07, 2.2e-07),  # 256
        (1.1e-07, 1.4e-07, 1.7e-07, 1.9e-07, 2.2e-07, 2.3e-07, 2.4e-07, 2.5e-07),  # 512
    ),
    ("smooth", "ppm4"): (
        (1.6e-07, 2.0e-07, 2.6e-07, 2.9e-07, 3.1e-07, 2.8e-07, 2.8e-07, 4.1e-07),  # 64
        (1.8e-07, 2.2e-07, 3.0e-07, 3.4e-07, 3.3e-07, 3.1e-07, 3.2e-07, 3.4e-07),  # 85
        (2.1e-07, 2.6e-07, 3.6e-07, 4.0e-07, 3.9e-07, 4.8e-07, 8.7e-07, 1.3e-05),  # 128
        (3.0e-07, 4.1e-07, 5.1e-07, 5.3e-07, 5.2e-07, 8.9e-07, 1.2e-06, 7.4e-05),  # 256
        (4.0e-07, 5.4e-07, 6.5e-07, 6.8e-07, 8.5e-07, 7.6e-06, 2.3e-05, 3.6e-05),  # 512
    ),
    ("smooth", "ppmx"): (
        (1.6e-07, 2.3e-07, 3.5e-07, 5.3e-07, 7.1e-06, 4.4e-05, 4.7e-05, 7.3e-05),  # 64
        (1.9e-07, 2.6e-07, 3.8e-07, 1.2e-06, 5.4e-06, 3.7e-05, 9.9e-05, 1.7e-04),  # 85
        (2.2e-07, 3.1e-07, 4.4e-07, 1.3e-06, 6.0e-06, 8.7e-05, 2.9e-04, 3.7e-04),  # 128
        (3.0e-07, 4.0e-07, 5.5e-07, 6.7e-07, 1.2e-05, 2.0e-04, 3.1e-04, 3.3e-04),  # 256
        (4.0e-07, 4.9e-07, 6.4e-07, 7.1e-07, 9.4e-06, 1.5e-04, 1.9e-04, 2.4e-04),  # 512
    ),
    ("smooth", "wenoz"): (
        (1.1e-07, 1.3e-07, 1.6e-07, 4.1e-07, 2.9e-06, 4.7e-05, 8.7e-05, 4.5e-04),  # 64
        (1.2e-07, 1.4e-07, 1.7e-07, 3.9e-06, 7.5e-05, 5.2e-04, 5.4e-04, 7.5e-04),  # 85
        (1.3e-07, 1.5e-07, 2.0e-07, 2.4e-06, 4.9e-05, 2.5e-04, 3.8e-04, 6.1e-04),  # 128
        (1.4e-07, 1.8e-07, 2.2e-07, 2.7e-07, 1.5e-05, 3.6e-04, 5.0e-04, 5.9e-04),  # 256
        (1.7e-07, 2.1e-07, 2.7e-07, 3.3e-07, 3.7e-05, 2.9e-04, 4.3e-04, 5.2e-04),  # 512
    ),
    ("turbulence", "dc"): (
        (5.5e-08, 6.7e-08, 6.6e-08, 7.4e-08, 7.7e-08, 3.9e-07, 2.1e-07, 1.6e-07),  # 64
        (5.9e-08, 6.1e-08, 6.9e-08, 7.1e-08, 7.3e-08, 7.5e-08, 8.0e-08, 8.0e-08),  # 85
        (6.0e-08, 6.1e-08, 6.3e-08, 7.2e-08, 7.4e-08, 7.0e-08, 8.4e-08, 8.6e-08),  # 128
        (6.7e-08, 6.7e-08, 7.6e-08, 7.6e-08, 8.6e-08, 1.1e-07, 1.7e-07, 1.4e-07),  # 256
        (8.4e-08, 8.3e-08, 9.5e-08, 9.8e-08, 1.1e-07, 1.1e-07, 1.2e-07, 1.2e-07),  # 512
    ),
    ("turbulence", "plm"): (
        (6.9e-08, 8.3e-08, 1.1e-07, 1.2e-07, 1.3e-07, 1.3e-07, 1.4e-07, 1.5e-07),  # 64
        (7.4e-08, 8.3e-08, 1.1e-07, 1.2e-07, 1.4e-07, 1.7e-06, 8.9e-05, 1.3e-04),  # 85
        (7.9e-08, 8.9e-08, 1.2e-07, 1.3e-07, 1.5e-07, 1.6e-07, 1.8e-07, 2.8e-05),  # 128
        (9.4e-08, 1.2e-07, 1.4e-07, 1.6e-07, 1.8e-07, 1.8e-07, 1.9e-07, 2.1e-07),  # 256
        (1.3e-07, 1.5e-07, 1.8e-07, 2.1e-07, 2.3e-07, 2.4e-07, 2.5e-07, 2.8e-07),  # 512
    ),
    ("turbulence", "ppm4"): (
        (1.2e-07, 1.6e-07, 2.1e-07, 2.4e-07, 2.8e-07, 3.0e-07, 3.6e-07, 6.0e-07),  # 64
        (1.4e-07, 1.8e-07, 2.4e-07, 4.9e-07, 3.6e-06, 3.6e-06, 4.5e-06, 7.8e-06),  # 85
        (1.8e-07, 2.3e-07, 3.1e-07, 3.7e-07, 4.6e-07, 7.0e-05, 8.3e-05, 1.1e-04),  # 128
        (2.5e-07, 3.4e-07, 4.4e-07, 5.3e-07, 6.2e-07, 6.5e-07, 6.6e-07, 7.0e-07),  # 256
        (3.6e-07, 4.7e-07, 7.6e-07, 1.3e-06, 1.4e-06, 1.5e-06, 1.3e-06, 1.1e-06),  # 512
    ),
    ("turbulence", "ppmx"): (
        (2.2e-07, 5.6e-07, 5.4e-06, 3.8e-05, 1.2e-04, 1.8e-04, 2.3e-04, 3.0e-04),  # 64
        (2.2e-07, 4.3e-07, 2.5e-06, 1.3e-05, 3.7e-05, 8.0e-05, 1.4e-04, 2.4e-04),  # 85
        (2.2e-07, 3.2e-07, 6.4e-07, 2.1e-06, 9.1e-06, 3.0e-05, 4.6e-05, 6.2e-05),  # 128
        (2.9e-07, 4.0e-07, 5.7e-07, 1.1e-05, 8.2e-06, 1.9e-05, 3.0e-05, 5.8e-05),  # 256
        (3.8e-07, 4.9e-07, 6.5e-07, 7.7e-07, 1.2e-06, 3.6e-06, 6.7e-06, 1.2e-05),  # 512
    ),
    ("turbulence", "wenoz"): (
        (9.9e-08, 1.3e-07, 1.5e-07, 1.8e-07, 2.2e-07, 2.4e-07, 2.6e-07, 2.6e-07),  # 64
        (1.1e-07, 1.3e-07, 1.7e-07, 2.0e-07, 2.3e-07, 3.1e-07, 5.1e-07, 2.7e-06),  # 85
        (1.2e-07, 1.5e-07, 1.8e-07, 2.2e-07, 2.6e-07, 2.7e-07, 5.3e-07, 1.8e-06),  # 128
        (1.5e-07, 1.8e-07, 2.3e-07, 2.7e-07, 3.0e-07, 3.3e-07, 3.5e-07, 3.8e-07),  # 256
        (1.9e-07, 2.2e-07, 2.8e-07, 3.4e-07, 3.7e-07, 4.1e-07, 4.4e-07, 5.9e-06),  # 512
    ),
}
# Float32 is kept where the estimate stays at or under FP32_ERR_BAR, five
# times below the 1e-5 L1 bar.
FP32_ERR_BAR = 2e-6


def fp32_error_estimate(problem, reconstruct, side, tlim):
    """Estimated float32-vs-float64 L1 density error of a request: the worst
    measured error (FP32_ERR) at any end time up to the first measured one
    at or past `tlim`, on the measured sides next to the request's (the side
    itself when measured, else the measured sides either side of it), times
    (side / 512)^2 above 512 (the measured growth on the shear layer is
    about 2-3x per doubling of the side at a fixed end time; 4x is the
    margin for unmeasured sides). None where nothing was measured (end
    times past 3, unknown problems)."""
    rows = FP32_ERR.get((problem, reconstruct))
    i = next((k for k, t in enumerate(FP32_ERR_TLIMS) if t >= tlim), None)
    if rows is None or i is None:
        return None
    above = next((k for k, s in enumerate(FP32_ERR_SIDES) if s >= side), len(FP32_ERR_SIDES) - 1)
    below = above if FP32_ERR_SIDES[above] <= side else max(above - 1, 0)
    worst = max(max(rows[k][:i + 1]) for k in {below, above})
    return worst * max(1.0, side / 512.0) ** 2


def served_dtype(req, dtype=None, guard=True):
    """The precision a request is served in: `dtype` if given, else the
    requested one, with float32 promoted to float64 where the guard's error
    estimate (fp32_error_estimate) is unknown or above FP32_ERR_BAR."""
    chosen = dtype or req.dtype
    if guard and chosen == "float32":
        est = fp32_error_estimate(req.problem, req.reconstruct, req.side, req.tlim)
        if est is None or est > FP32_ERR_BAR:
            return "float64"
    return chosen


def _device_state(problem, n):
    """The request's initial state built on the device in float64 (the
    formulas of initial_conditions.kelvin_helmholtz_tanh, smooth_waves and
    uniform_rest, evaluated by torch instead of NumPy)."""
    t = _lib.torch()
    dev = _lib.device()
    c = (t.arange(n, dtype=t.float64, device=dev) + 0.5) / n - 0.5
    Y, X = t.meshgrid(c, c, indexing="ij")
    if problem == "kh":
        inside = 0.5 * (t.tanh((Y + 0.25) / 0.01) - t.tanh((Y - 0.25) / 0.01))
        vy = 0.01 * t.sin(4 * t.pi * X) * (t.exp(-((Y - 0.25) / 0.05) ** 2) + t.exp(-((Y + 0.25) / 0.05) ** 2))
        return t.stack((t.ones_like(X), inside - 0.5, vy, inside), dim=-1)
    if problem == "smooth":
        px, py = 2.0 * t.pi * X, 2.0 * t.pi * Y
        rho = 1.0 + 0.1 * t.sin(px + py)
        return t.stack((rho, rho * (0.2 * t.cos(py)), rho * (0.2 * t.sin(px))), dim=-1)
    U = t.zeros((n, n, 3), dtype=t.float64, device=dev)
    U[..., 0] = 1.0
    return U


def warmup_requests(dtypes=("float32", "float64"), sides=(16,)):
    """One short request per problem, reconstruction, Riemann solver,
    precision and side: running them once loads every kernel a stream can use
    (CUDA loads kernels lazily, at their first launch), so a server's first
    requests do not pay for it. With tuned tiles the size classes run
    different kernels, so a server warms one side per class."""
    out = []
    for side in sides:
        for dtype in dtypes:
            for problem in PROBLEMS:
                for recon in RECONS:
                    for rsolver in SOLVERS:
                        out.append(Request(rid=-1 - len(out), arrival=0.0, problem=problem, side=side,
                                           reconstruct=recon, rsolver=rsolver, tlim=0.004 * 16 / side, dtype=dtype,
                                           seed=1))
    return out


def build_solve(req, tile=None, clock=None, dtype=None):
    """The device-resident Solve of one request (the reference's problem set-ups, run.py:133-163).

    ``tile`` None picks :data:`SERVING_TILES` by precision.
    """
    t = _lib.torch()
    from .forcing import cartesian_modes, forcing_basis, modal_coefficients
    from .initial_conditions import cell_centers
    from .solver import Solve
    n = req.side
    dtype = dtype or req.dtype
    kw = dict(reconstruct=req.reconstruct, rsolver=req.rsolver,
              tile=tuple(tile) if tile is not None else SERVING_TILES[dtype],
              dtype=getattr(t, dtype), clock=clock)
    U0 = _device_state(req.problem, n)
    if req.problem == "kh":
        return Solve(U0, 1 / n, 1 / n, 1.0, 1e-10, "rk3", 0.4, req.tlim, 10**7, **kw)
    if req.problem == "smooth":
        return Solve(U0, 1 / n, 1 / n, 1.0, 1e-10, "rk3", 0.4, req.tlim, 10**7, **kw)
    x, _ = cell_centers(n, n)
    modes = cartesian_modes(3, 5, (-5, 5), (-5, 5))
    updates = int(np.ceil(req.tlim / 0.0075)) + 1
    table = modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, req.seed, 0.75, 0.0075, updates)
    basis = forcing_basis(modes, x, x, (1.0, 1.0))
    return Solve(U0, 1 / n, 1 / n, 1.0, 1.17549e-38, "rk3", 0.4, req.tlim, 10**7,
                 viscosity=1.5e-6, drag_rate=0.3333335, forcing=(table, basis), dt_update=0.0075,
                 dedt=0.03703705, **kw)


def footprint_bytes(req, dtype=None):
    """Device bytes a request holds while live (states, workspace, forcing tables)."""
    nvar = 4 if req.problem == "kh" else 3
    w = 4 if (dtype or req.dtype) == "float32" else 8
    cells = req.side * req.side
    states = 3 * cells * nvar * w
    workspace = (cells // (32 * 8) + 4096) * 32 + 64 * 1024
    forcing = 0
    if req.problem == "turbulence":
        updates = int(np.ceil(req.tlim / 0.0075)) + 1
        forcing = updates * 56 * 32 + 4 * 56 * req.side * w + cells * 2 * w
    return states + workspace + forcing


class Server:
    """Continuous-batching request loop with an HBM admission budget.

    ``tile``: a fixed stage tile for every request, None for SERVING_TILES,
    or "auto" (default): the autotuner's choice per (precision, size class,
    reconstruction), tuned on probe grids the first time such a request is
    built (cached per GPU model; :meth:`warmup` tunes every class up front).
    ``guard``: serve float32 requests in float64 where served_dtype's error estimate says.
    """

    def __init__(self, budget_bytes=150e9, tile="auto", steps_per_tick=4, blocks_per_sm=0,
                 max_live=1024, keep_results=False, dtype=None, builder=None, guard=True):
        self.budget = float(budget_bytes)
        self.tile = tile
        self.steps_per_tick = steps_per_tick
        self.blocks_per_sm = blocks_per_sm
        self.max_live = max_live
        self.keep_results = keep_results
        self.dtype = dtype  # serve every request in this precision (None: as requested)
        self.guard = guard
        self.builder = builder or build_solve  # (request, tile, clock, dtype) -> Solve
        self.tuned = {}  # (precision, size class, reconstruction) -> autotune result

    def dtype_for(self, req):
        return served_dtype(req, self.dtype, self.guard)

    def tile_for(self, req):
        """The stage tile request `req` is served with."""
        if self.tile != "auto":
            return tuple(self.tile) if self.tile is not None else SERVING_TILES[self.dtype_for(req)]
        dtype = self.dtype_for(req)
        key = (dtype, size_class(req.side), req.reconstruct)
        if key not in self.tuned:
            from . import autotune
            _, side, count = SIZE_CLASSES[key[1]]
            self.tuned[key] = autotune.tune(dtype, req.reconstruct, "roe", 4, side, count=count)
        return tuple(self.tuned[key]["tile"])

    def tile_table(self):
        """{"float32/class0/ppm4": {"tile": [...], "knobs": {...}}, ...} of the tiles tuned so far."""
        return {f"{d}/class{c}/{r}": {"tile": v["tile"], "knobs": v["knobs"]}
                for (d, c, r), v in sorted(self.tuned.items())}

    def warmup(self):
        """Serve :func:`warmup_requests` once (untimed) to load every kernel
        and, with automatic tiles, tune every size class and reconstruction,
        in every precision a request can be served in (float64 too where the
        guard may promote float32 requests)."""
        dtypes = (self.dtype,) if self.dtype else ("float32", "float64")
        if self.guard and "float32" in dtypes and "float64" not in dtypes:
            dtypes += ("float64",)
        if self.tile == "auto":
            for dtype in dtypes:
                for top, side, _ in SIZE_CLASSES:
                    for recon in RECONS:
                        self.tile_for(Request(rid=-1, arrival=0.0, problem="kh", side=min(top, side),
                                              reconstruct=recon, rsolver="roe", tlim=0.0, dtype=dtype, seed=1))
        # One side per size class (its smallest) where the classes' tiles differ.
        sides = (16,) if self.tile != "auto" else (16,) + tuple(top + 1 for top, _, _ in SIZE_CLASSES[:-1])
        forced, self.dtype = self.dtype, None  # each warm-up request in its own precision
        try:
            self.run(warmup_requests(dtypes, sides))
        finally:
            self.dtype = forced

    def run(self, requests):
        """Serve `requests` (arrival-ordered or not); returns a stats dict.

        The loop is pipelined: each tick enqueues its steps and a snapshot of
        every clock, then reads the previous tick's snapshot while the GPU
        runs this one. Solves found finished are retired (box sums for the
        failure check and, with keep_results, the state copied to pinned host
        memory, all stream-ordered) and leave the next plan; their memory and
        clock slot return once those copies have landed. Completion times
        are the GPU time of the snapshot that first showed the solve done.
        """
        t = _lib.torch()
        from .batch import Batch, ClockBank
        bank = ClockBank(self.max_live)
        sums_dev = t.empty((self.max_live, 4), dtype=t.float64, device=_lib.device())
        sums_host = t.empty((self.max_live, 4), dtype=t.float64).pin_memory()
        free_slots = list(range(self.max_live - 1, -1, -1))
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        live = []          # (req, solve, slot)
        retiring = []      # (req, solve, slot, event, result_host, clock)
        in_use = 0.0
        batch = None
        changed = True
        ticks = 0
        peak_live = 0
        peak_bytes = 0.0
        previous = None    # (event, host clocks, live list) of the last tick
        t.cuda.synchronize()
        start = t.cuda.Event(enable_timing=True)
        start.record()
        t0 = time.perf_counter()

        def finish(entry, wait):
            req, solve, slot, event, result_host, c = entry
            if not (wait or event.query()):
                return False
            event.synchronize()
            sums = sums_host[slot, :solve.desc.nvar].numpy()
            # A non-finite state drives dt to NaN and stops the solve early
            # (run.py:178-180 raises there); a tracer-only NaN leaves dt
            # finite, so the box sums are checked as well.
            if not (c.time == c.tlim or c.cycle >= c.nlim) or not np.isfinite(c.time) \
                    or not np.all(np.isfinite(sums)):
                req.error = f"stopped at t={c.time} after {c.cycle} steps (non-finite state)"
            elif result_host is not None:
                req.result = result_host.numpy()
            free_slots.append(slot)
            return True

        while pending or live or retiring or previous:
            now = time.perf_counter() - t0
            while (pending and pending[0].arrival <= now and free_slots
                   and in_use + footprint_bytes(pending[0], self.dtype_for(pending[0])) <= self.budget):
                req = pending.popleft()
                slot = free_slots.pop()
                req.served_dtype = self.dtype_for(req)
                solve = self.builder(req, self.tile_for(req), clock=bank.slot(slot), dtype=req.served_dtype)
                req.admitted = time.perf_counter() - t0
                live.append((req, solve, slot))
                in_use += footprint_bytes(req, req.served_dtype)
                peak_bytes = max(peak_bytes, in_use)
                changed = True
            current = None
            if live:
                if changed:
                    batch = Batch([s for _, s, _ in live], blocks_per_sm=self.blocks_per_sm)
                    changed = False
                for _ in range(self.steps_per_tick):
                    batch.enqueue_step()
                ticks += 1
                peak_live = max(peak_live, len(live))
                event, host = bank.snapshot()
                current = (event, host, list(live))
            # Retirements whose copies have landed free their memory and slot.
            keep = []
            for entry in retiring:
                if finish(entry, wait=not live and previous is None):
                    in_use -= footprint_bytes(entry[0], entry[0].served_dtype)
                else:
                    keep.append(entry)
            retiring = keep
            if previous is not None:
                event, host, members = previous
                event.synchronize()  # the GPU keeps running the tick just enqueued
                stamp = start.elapsed_time(event) * 1e-3
                clocks = bank.parse(host)
                # Members already retired from an earlier snapshot are skipped.
                still = {id(solve) for _, solve, _ in live}
                done = {slot for _, solve, slot in members if id(solve) in still and clocks[slot].done}
                if done:
                    for req, solve, slot in members:
                        if slot not in done or id(solve) not in still:
                            continue
                        req.finished = stamp
                        req.cycles = clocks[slot].cycle
                        nv = solve.desc.nvar
                        _lib.call("jx_box_sums", ctypes.byref(solve.desc), _lib.ptr(solve.S),
                                  _lib.ptr(sums_dev[slot]), _lib.ptr(solve.ws), solve.nbytes,
                                  _lib.stream_handle())
                        sums_host[slot, :nv].copy_(sums_dev[slot, :nv], non_blocking=True)
                        result_host = None
                        if self.keep_results:
                            result_host = t.empty(solve.S.shape, dtype=solve.S.dtype).pin_memory()
                            result_host.copy_(solve.S, non_blocking=True)
                        copied = t.cuda.Event()
                        copied.record()
                        retiring.append((req, solve, slot, copied, result_host, clocks[slot]))
                    live = [e for e in live if e[2] not in done]
                    changed = True
            previous = current
            if not live and not retiring and pending and previous is None:
                wait = pending[0].arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(min(wait, 0.01))
                elif in_use + footprint_bytes(pending[0], self.dtype_for(pending[0])) > self.budget:
                    raise RuntimeError(f"request {pending[0].rid} does not fit in the HBM budget")
        t.cuda.synchronize()
        elapsed = time.perf_counter() - t0
        ok = [r for r in requests if r.error is None]
        tts = np.array([r.finished - r.arrival for r in ok]) if ok else np.array([np.nan])
        return {
            "requests": len(requests), "completed": len(ok), "failed": len(requests) - len(ok),
            "elapsed_s": elapsed, "solves_per_s": len(ok) / elapsed,
            "tts_p50_s": float(np.percentile(tts, 50)), "tts_p99_s": float(np.percentile(tts, 99)),
            "ticks": ticks, "peak_live": peak_live, "peak_bytes": peak_bytes,
        "promoted_to_float64": sum(1 for r in requests if r.served_dtype != (self.dtype or r.dtype)),
        }


def run_serial(requests, dtype="float64", keep_results=False):
    """The baseline: each request alone, one after another, in `dtype`."""
    t = _lib.torch()
    t.cuda.synchronize()
    t0 = time.perf_counter()
    for req in requests:
        solve = build_solve(req, dtype=dtype)
        solve.run(steps_per_sync=32)
        req.cycles = solve.state().cycle
        if keep_results:
            req.result = solve.S.cpu().numpy()
        del solve
    t.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    return {"requests": len(requests), "elapsed_s": elapsed, "solves_per_s": len(requests) / elapsed}
