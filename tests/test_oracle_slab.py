"""The row-slab driver of the float64 oracle (the CPU baseline on the
benchmark's whole grid) reproduces the oracle's whole-grid evolve cycles bit
for bit: even and uneven slabs, every integrator, two methods."""

import numpy as np
import pytest

from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
from oracle import hydro_oracle as H
from oracle import slab


def whole_grid(U, cycles, recon, solver, integrator):
    n = U.shape[0]
    prev = np.inf
    for _ in range(cycles):
        _, W = H.primitives(U, 1e-10)
        dt = float(H.timestep(W, 1 / n, 1 / n, 1.0, 0.4, prev, 0.0, 1e30))
        U = H.step(U, dt, 1 / n, 1 / n, 1.0, 1e-10, integrator, recon=recon, solver=solver)
        prev = dt
    return U


@pytest.mark.parametrize("n,procs,recon,solver,integrator", [
    (48, 4, "ppm4", "roe", "rk3"),
    (50, 3, "wenoz", "hlle", "rk2"),
    (40, 5, "ppmx", "llf", "rk4"),
])
def test_slabs_match_whole_grid_bitwise(n, procs, recon, solver, integrator):
    U0 = kelvin_helmholtz_tanh(n, n)
    out, seconds, used = slab.run(U0, cycles=2, procs=procs, warm=1, recon=recon, solver=solver,
                                  integrator=integrator)
    assert used == procs and seconds > 0
    np.testing.assert_array_equal(out, whole_grid(U0, 3, recon, solver, integrator))


def test_slab_bounds_cover_the_grid():
    for n, procs in ((4096, 16), (50, 3), (7, 7)):
        bounds = [slab.slab_bounds(n, procs, r) for r in range(procs)]
        assert bounds[0][0] == 0 and bounds[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(bounds, bounds[1:]))


def test_a_failing_worker_is_reported_not_waited_for():
    U0 = kelvin_helmholtz_tanh(24, 24)
    with pytest.raises(RuntimeError, match="failed"):
        slab.run(U0, cycles=1, procs=2, recon="no-such-method")
