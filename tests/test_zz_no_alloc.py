"""jx_timestep_noalloc, the timestep entry point that allocates nothing.

It exists for callers that cannot allocate device memory and have no
workspace to hand over: a JAX/XLA FFI handler (XLA reserves most of the GPU
up front and owns every buffer, so a cudaMalloc inside a handler can fail and
would also synchronise the device), or a time loop that forbids allocation
after start-up. Its scratch is a static 65,792-byte array inside libjx.so.

The test calls it through the C ABI twice in a row, first on a large grid and
then on a much smaller one (so a count left over from the first call would
corrupt the second), and each time compares the result with jx_timestep,
which takes a caller-owned workspace. This file sorts last so that a run that
stops at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest
from conftest import STEP_RTOL, assert_rel

pytestmark = pytest.mark.gpu


def primitives(ny, nx, seed):
    rng = np.random.default_rng(seed)
    W = np.empty((ny, nx, 4))
    W[..., 0] = 1.0 + rng.random((ny, nx))
    W[..., 1:] = rng.standard_normal((ny, nx, 3))
    return W


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_timestep_noalloc_matches_workspace_entry_point(dtype):
    import torch
    from jathenax_gb300 import _lib
    from jathenax_gb300.hydro import make_desc

    cases = [  # (ny, nx, seed, cfl, prev_dt, time, tlim, viscosity, smagorinsky_cs, drag)
        (1536, 1024, 1, 0.4, np.inf, 0.0, 1.0, 1e-3, 0.17, 0.3),
        (6, 8, 2, 0.4, 1e-4, 0.0, 1.0, 0.0, 0.0, 0.0),
    ]
    stream = _lib.stream_handle()
    for ny, nx, seed, cfl, prev_dt, time, tlim, nu, cs_smag, drag in cases:
        W = torch.as_tensor(primitives(ny, nx, seed), device="cuda").to(getattr(torch, dtype))
        desc = make_desc(W.shape, W.dtype, 1 / nx, 1 / ny, 1.0, 1e-10, viscosity=nu,
                         smagorinsky_cs=cs_smag, drag_rate=drag)
        ws, nbytes = _lib.workspace(desc)
        expected = torch.empty(1, dtype=torch.float64, device="cuda")
        got = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        _lib.call("jx_timestep", ctypes.byref(desc), _lib.ptr(W), cfl, prev_dt, time, tlim,
                  _lib.ptr(expected), _lib.ptr(ws), nbytes, stream)
        _lib.call("jx_timestep_noalloc", ctypes.byref(desc), _lib.ptr(W), cfl, prev_dt, time, tlim,
                  _lib.ptr(got), stream)
        torch.cuda.synchronize()
        assert np.isfinite(got.item())
        assert_rel(got.item(), expected.item(), STEP_RTOL, f"{ny}x{nx} {dtype}")


def test_timestep_noalloc_rejects_bad_arguments():
    from jathenax_gb300 import _lib
    from jathenax_gb300.hydro import make_desc
    desc = make_desc((6, 8, 3), "float64", 1 / 8, 1 / 6, 1.0, 1e-10)
    status = _lib.load().jx_timestep_noalloc(ctypes.byref(desc), None, 0.4, np.inf, 0.0, 1.0, None,
                                             _lib.stream_handle())
    assert status == _lib.JX_ERR_INVALID
    assert b"null" in _lib.load().jx_last_error()
