"""The register-marching stage kernel (58-column tiles) against the
shared-memory tile kernel (32-column tiles) and the float64 oracle; one and
three columns per lane (26- and 90-column tiles) against two.

Both kernels evaluate every face and cell with the same device functions in
the same order; where they can still differ is the compiler's contraction of
a multiply and an add into one FMA, which depends on how often a product is
reused (with donor-cell edges the x and y Riemann problems of a cell share
products). So the two kernels are compared at the step tolerance in float64
(in float32: 1e-6 in L1 per component and 1e-3 of each component's largest
magnitude pointwise), over every
reconstruction and Riemann solver, the viscous, drag and SGS-stress terms,
RK4's saved-register stages and ragged and tiny periodic grids (fewer cells
than one strip or one tile); the marching kernel against itself is bitwise
for every tile height and every column count per lane.
"""

import numpy as np
import pytest
from conftest import STEP_RTOL, assert_rel

from oracle import hydro_oracle as H
from test_gpu_parity import RECONS, SOLVERS, noisy_state

pytestmark = pytest.mark.gpu


def stepped(U0, dtype, tile, integrator="rk3", steps=1, dt=0.001, recon="ppm4", rsolver="roe", tau=None,
            **kw):
    import torch
    from jathenax_gb300 import _lib
    from jathenax_gb300 import hydro as G
    ny, nx = U0.shape[:2]
    desc = G.make_desc(U0.shape, dtype, 1 / nx, 1 / ny, 1.0, 1e-10, integrator, reconstruct=recon,
                       rsolver=rsolver, tile=tile, **kw)
    ws, nbytes = _lib.workspace(desc)
    U = torch.as_tensor(U0, device="cuda").to(dtype)
    predict = None
    if tau is not None:
        T = torch.as_tensor(tau, device="cuda").to(dtype)
        predict = lambda w, W: w * T  # noqa: E731 - a fixed stress field
    for _ in range(steps):
        clock = _lib.new_clock(dt=dt)
        U, _ = G.run_stages(desc, U, clock=clock, ws=ws, nbytes=nbytes, predict_stress=predict,
                            sgs_weights=torch.ones((), device="cuda", dtype=dtype) if tau is not None else None)
    return U.cpu().numpy()


def assert_close(a, b, what):
    if a.dtype == np.float64:
        assert_rel(a, b, STEP_RTOL, what)
        return
    # float32: a rounding-level difference may flip a limiter branch (PPMX's
    # smooth-extremum test, WENO-Z's near-flat weights) in a cell or two of a
    # noisy state, so the pointwise bound is looser than the grid average.
    assert_rel(a, b, 1e-3, what)
    l1 = np.abs(a.astype(np.float64) - b).mean(axis=(0, 1)) / np.abs(b.astype(np.float64)).mean(axis=(0, 1))
    assert l1.max() <= 1e-6, f"{what}: L1 difference {l1.max():.2e}"


def assert_bitwise(a, b, what):
    assert a.dtype == b.dtype and a.shape == b.shape, what
    same = a.view(np.uint8).reshape(a.shape + (-1,)) == b.view(np.uint8).reshape(b.shape + (-1,))
    bad = np.argwhere(~np.all(same, axis=-1))
    assert len(bad) == 0, f"{what}: {len(bad)} values differ, first at {bad[:3].tolist()}"


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("rs", SOLVERS)
@pytest.mark.parametrize("rec", RECONS)
def test_marching_matches_tile_kernel(rec, rs, dtype):
    import torch
    U0 = noisy_state(213, 77, nvar=4, seed=RECONS.index(rec) * 3 + SOLVERS.index(rs))
    td = getattr(torch, dtype)
    a = stepped(U0, td, (58, 16), recon=rec, rsolver=rs, steps=2)
    b = stepped(U0, td, (32, 16), recon=rec, rsolver=rs, steps=2)
    assert_close(a, b, f"{rec}/{rs}/{dtype}")


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("integrator", ["rk2", "rk4"])
def test_marching_viscous_drag_three_variables(integrator, dtype):
    import torch
    U0 = noisy_state(150, 61, nvar=3, seed=4)
    td = getattr(torch, dtype)
    kw = dict(viscosity=2e-3, smagorinsky_cs=0.2, drag_rate=0.3)
    a = stepped(U0, td, (58, 12), integrator=integrator, rsolver="hlle", **kw)
    b = stepped(U0, td, (32, 8), integrator=integrator, rsolver="hlle", **kw)
    assert_close(a, b, f"{integrator}/{dtype}")


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_marching_sgs_stress(dtype):
    import torch
    U0 = noisy_state(120, 40, nvar=4, seed=8)
    tau = 1e-3 * np.random.default_rng(3).standard_normal((40, 120, 3))
    td = getattr(torch, dtype)
    a = stepped(U0, td, (58, 8), recon="wenoz", tau=tau)
    b = stepped(U0, td, (32, 16), recon="wenoz", tau=tau)
    assert_close(a, b, dtype)


@pytest.mark.parametrize("shape", [(5, 7), (1, 40), (33, 1), (9, 59), (9, 105), (70, 26), (64, 116)])
def test_marching_tiny_and_ragged_grids(shape):
    import torch
    ny, nx = shape
    U0 = noisy_state(nx, ny, nvar=4, seed=ny + nx)
    for rec in ("ppm4", "wenoz", "plm", "dc"):
        a = stepped(U0, torch.float64, (58, 8), recon=rec)
        b = stepped(U0, torch.float64, (32, 16), recon=rec)
        assert_close(a, b, f"{shape} {rec}")
        ref = H.step(U0, 0.001, 1 / nx, 1 / ny, 1.0, 1e-10, "rk3", recon=rec)
        assert_rel(a, ref, STEP_RTOL, f"{shape} {rec} vs oracle")


def test_marching_tile_height_does_not_change_results():
    import torch
    U0 = noisy_state(300, 190, nvar=4, seed=12)
    base = stepped(U0, torch.float32, (58, 8), steps=3)
    for rows in (12, 16, 24, 32, 48, 64, 100):
        assert_bitwise(stepped(U0, torch.float32, (58, rows), steps=3), base, f"rows {rows}")
    # The automatic tile (device-dependent height) gives the same state too.
    assert_bitwise(stepped(U0, torch.float32, (0, 0), steps=3), base, "automatic tile")


@pytest.mark.parametrize("rs", SOLVERS)
@pytest.mark.parametrize("rec", RECONS)
def test_columns_per_lane_do_not_change_results(rec, rs):
    """Float32, lean (inviscid) forms: 1, 2 and 3 columns per lane, bitwise."""
    import torch
    U0 = noisy_state(187, 70, nvar=4, seed=RECONS.index(rec) * 3 + SOLVERS.index(rs) + 40)
    base = stepped(U0, torch.float32, (58, 16), recon=rec, rsolver=rs, steps=2)
    # 24 rows and more: the cp.async row ring where it is built.
    for tile in ((26, 16), (90, 12), (26, 24), (58, 40), (90, 28)):
        assert_bitwise(stepped(U0, torch.float32, tile, recon=rec, rsolver=rs, steps=2), base, f"{rec}/{rs} {tile}")


@pytest.mark.parametrize("integrator", ["rk2", "rk4"])
def test_columns_per_lane_viscous_drag_and_stress(integrator):
    """Float32, generic form (viscosity, Smagorinsky, drag, SGS stress, RK4's
    saved register), ragged grid: 1, 2 and 3 columns per lane, bitwise."""
    import torch
    U0 = noisy_state(131, 45, nvar=3, seed=9)
    kw = dict(viscosity=2e-3, smagorinsky_cs=0.2, drag_rate=0.3)
    tau = 1e-3 * np.random.default_rng(5).standard_normal((45, 131, 3))
    base = stepped(U0, torch.float32, (58, 12), integrator=integrator, rsolver="hlle", tau=tau, **kw)
    for tile in ((26, 8), (90, 20), (26, 30), (58, 24), (90, 45)):
        got = stepped(U0, torch.float32, tile, integrator=integrator, rsolver="hlle", tau=tau, **kw)
        assert_bitwise(got, base, f"{integrator} {tile}")


@pytest.mark.parametrize("shape", [(5, 7), (1, 40), (9, 27), (9, 91), (70, 26), (64, 181)])
def test_columns_per_lane_on_tiny_and_ragged_grids(shape):
    import torch
    ny, nx = shape
    U0 = noisy_state(nx, ny, nvar=4, seed=ny * nx)
    for rec in ("ppm4", "wenoz"):
        base = stepped(U0, torch.float32, (58, 8), recon=rec)
        for tile in ((26, 8), (90, 8), (26, 24), (58, 32)):
            assert_bitwise(stepped(U0, torch.float32, tile, recon=rec), base, f"{shape} {rec} {tile}")


@pytest.mark.parametrize("rs", SOLVERS)
@pytest.mark.parametrize("rec", RECONS)
def test_float32_kernel_families_are_bitwise_equal(rec, rs):
    """Float32 rounds every operation explicitly, so the shared-memory tile
    kernel and the marching kernel give the same bits (float64 agrees to the
    step tolerance only; see test_marching_matches_tile_kernel)."""
    import torch
    U0 = noisy_state(150, 66, nvar=4, seed=RECONS.index(rec) * 3 + SOLVERS.index(rs) + 70)
    a = stepped(U0, torch.float32, (58, 16), recon=rec, rsolver=rs, steps=2)
    b = stepped(U0, torch.float32, (32, 16), recon=rec, rsolver=rs, steps=2)
    assert_bitwise(a, b, f"{rec}/{rs}")
    kw = dict(viscosity=2e-3, smagorinsky_cs=0.2, drag_rate=0.3)
    a = stepped(U0[..., :3], torch.float32, (26, 12), recon=rec, rsolver=rs, integrator="rk4", **kw)
    b = stepped(U0[..., :3], torch.float32, (32, 8), recon=rec, rsolver=rs, integrator="rk4", **kw)
    assert_bitwise(a, b, f"{rec}/{rs} viscous rk4")
