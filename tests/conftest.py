import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

# Parity bar for the float64 kernels against the float64 oracle: the largest
# per-component error over the grid, relative to that component's largest
# magnitude, after one stage or step (the kernels contract FMAs and multiply
# by reciprocals of loop constants, so they differ from NumPy at the ulp level).
STEP_RTOL = 1e-12
# After a whole run.
RUN_RTOL = 1e-10


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libjx.so")


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def load(name):
        if name not in cache:
            with np.load(GOLDEN / f"{name}.npz") as data:
                cache[name] = {k: data[k] for k in data.files}
        return cache[name]
    return load


def max_rel_error(actual, expected):
    """Largest |a - e| per trailing component, over max |e| of that component."""
    a = np.asarray(actual, dtype=np.float64)
    e = np.asarray(expected, dtype=np.float64)
    assert a.shape == e.shape, (a.shape, e.shape)
    if a.ndim == 0:
        return abs(float(a - e)) / max(abs(float(e)), 1e-300)
    a2 = a.reshape(-1, a.shape[-1]) if a.ndim > 1 else a.reshape(-1, 1)
    e2 = e.reshape(-1, e.shape[-1]) if e.ndim > 1 else e.reshape(-1, 1)
    scale = np.maximum(np.max(np.abs(e2), axis=0), 1e-300)
    return float(np.max(np.max(np.abs(a2 - e2), axis=0) / scale))


def assert_rel(actual, expected, tol, what=""):
    err = max_rel_error(actual, expected)
    assert err <= tol, f"{what}: max relative error {err:.3e} > {tol:.1e}"
