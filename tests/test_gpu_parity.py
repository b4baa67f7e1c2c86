"""GPU kernels (through the C ABI) against the float64 CPU oracle.

Tolerances: one stage/step <= 1e-12 and a whole run <= 1e-10, relative to
each component's largest magnitude (conftest.STEP_RTOL / RUN_RTOL). CFL dt
selection is bitwise (the kernel reduces exactly). FP32 state is checked
against the FP64 oracle at 1e-5.
"""

import numpy as np
import pytest
from conftest import RUN_RTOL, STEP_RTOL, assert_rel, max_rel_error

from oracle import forcing_oracle as F
from oracle import hydro_oracle as H
from oracle import run_oracle as R

pytestmark = pytest.mark.gpu

RECONS = ("dc", "plm", "ppm4", "ppmx", "wenoz")
SOLVERS = ("llf", "hlle", "roe")
INTEGRATORS = ("rk2", "rk3", "rk4")


def noisy_state(nx, ny, nvar=4, seed=0, amplitude=0.05):
    rng = np.random.default_rng(seed)
    x, y = R.cell_centers(nx, ny)
    X, Y = np.meshgrid(x, y)
    rho = 1.0 + 0.3 * np.sin(2 * np.pi * (X + 2 * Y)) + 0.2 * rng.random((ny, nx))
    vx = 0.6 * np.tanh(np.cos(2 * np.pi * Y) / 0.1) + amplitude * rng.standard_normal((ny, nx))
    vy = 0.3 * np.sin(4 * np.pi * X) + amplitude * rng.standard_normal((ny, nx))
    comps = [rho, rho * vx, rho * vy]
    for k in range(nvar - 3):
        comps.append(rho * (0.5 + 0.5 * np.sin(2 * np.pi * (k + 1) * X) * np.cos(2 * np.pi * Y)))
    return np.stack(comps, axis=-1)


@pytest.fixture(scope="module")
def G():
    from jathenax_gb300 import hydro
    return hydro


@pytest.mark.parametrize("integ", INTEGRATORS)
@pytest.mark.parametrize("rs", SOLVERS)
@pytest.mark.parametrize("rec", RECONS)
def test_step_matches_oracle(G, rec, rs, integ):
    U0 = noisy_state(45, 37, seed=RECONS.index(rec) * 9 + SOLVERS.index(rs) * 3 + INTEGRATORS.index(integ))
    args = (0.002, 1 / 45, 1 / 37, 1.0, 1e-10, integ)
    gpu = G.isothermal_step(U0, *args, reconstruct=rec, rsolver=rs)
    ref = H.step(U0, *args, recon=rec, solver=rs)
    assert_rel(gpu, ref, STEP_RTOL, f"{rec}/{rs}/{integ}")


@pytest.mark.parametrize("rs", SOLVERS)
def test_viscous_smagorinsky_drag_step(G, rs):
    U0 = noisy_state(40, 24, nvar=3, seed=5)
    args = (0.002, 1 / 40, 1 / 24, 1.0, 1e-10, "rk3")
    kw = dict(viscosity=2e-3, smagorinsky_cs=0.2, drag_rate=0.3)
    gpu = G.isothermal_step(U0, *args, rsolver=rs, **kw)
    ref = H.step(U0, *args, solver=rs, nu=2e-3, cs_smag=0.2, drag=0.3)
    assert_rel(gpu, ref, STEP_RTOL)


@pytest.mark.parametrize("pair", [("ppm4", "roe"), ("ppmx", "llf"), ("wenoz", "hlle"), ("plm", "roe")])
@pytest.mark.parametrize("integ", INTEGRATORS)
def test_stage_traces_match_oracle(G, pair, integ):
    rec, rs = pair
    U0 = noisy_state(34, 18, nvar=5, seed=11)
    args = (0.003, 1 / 34, 1 / 18, 1.0, 1e-10, integ)
    _, gpu = G.isothermal_step(U0, *args, viscosity=1e-3, smagorinsky_cs=0.1, reconstruct=rec,
                               rsolver=rs, trace=True)
    _, ref = H.step(U0, *args, nu=1e-3, cs_smag=0.1, recon=rec, solver=rs, trace=True)
    assert len(gpu) == len(ref)
    for number, (a, b) in enumerate(zip(gpu, ref), 1):
        for field in H_TRACE_FIELDS:
            assert_rel(a[field], b[field], STEP_RTOL, f"stage {number} {field}")


H_TRACE_FIELDS = ("primitives", "left_x", "right_x", "left_y", "right_y", "flux_x", "flux_y",
                  "saved", "conserved")


def test_golden_step_fixture(G, golden):
    g = golden("steps")
    for rec in RECONS:
        for rs in SOLVERS:
            for integ in INTEGRATORS:
                gpu = G.isothermal_step(g["U0"], 0.004, 1 / 12, 1 / 10, 1.0, 1e-10, integ,
                                        reconstruct=rec, rsolver=rs)
                assert_rel(gpu, g[f"{rec}_{rs}_{integ}"], STEP_RTOL, f"{rec}/{rs}/{integ}")


def test_forced_step_and_kick_trace(G, golden):
    g = golden("forcing")
    U = g["U"]
    kicked, stages = G.isothermal_step(U, 0.003, 1 / 16, 1 / 12, 1.0, 1e-10, "rk3", viscosity=1e-3,
                                       drag_rate=0.3, raw_force=g["raw"], dedt=0.04, trace=True)
    assert_rel(kicked, g["kicked"], STEP_RTOL, "kicked")
    assert_rel(stages[-1]["before_kick"], g["before_kick"], STEP_RTOL, "before_kick")
    assert_rel(stages[-1]["acceleration"], g["kick_acceleration"], STEP_RTOL, "acceleration")


def test_normalize_and_render_force(golden):
    from jathenax_gb300 import forcing as GF
    g = golden("forcing")
    accel = GF.normalize_force(g["U"], g["raw"], 0.003, 0.04)
    assert_rel(accel, g["acceleration"], STEP_RTOL)
    basis = GF.forcing_basis(g["modes"], g["x"], g["y"], (1.0, 1.0))
    raw = GF.render_force(g["table"][2], basis).cpu().numpy()
    assert_rel(raw, g["raw"], STEP_RTOL)
    assert np.all(GF.normalize_force(g["U"], g["raw"], 0.003, 0.0) == 0.0)


def test_sgs_hook_matches_reference_fixture(G, golden):
    import torch
    g = golden("sgs")
    weights = torch.as_tensor(g["scale"], device="cuda")
    calls = []

    def predict_stress(w, W):
        calls.append(tuple(W.shape))
        return w * W

    final, stages = G.isothermal_step(g["U"], 0.01, 1 / 8, 1 / 8, 1.0, 1e-10, "rk3", trace=True,
                                      predict_stress=predict_stress, sgs_weights=weights)
    assert calls == [(8, 8, 3)] * 3
    assert_rel(final, g["final"], STEP_RTOL)
    for number, stage in enumerate(stages, 1):
        assert_rel(stage["flux_x"], g[f"s{number}_flux_x"], STEP_RTOL)
        assert_rel(stage["flux_y"], g[f"s{number}_flux_y"], STEP_RTOL)


def test_timestep_selection_is_exact(golden):
    from jathenax_gb300.hydro import isothermal_timestep
    g = golden("timestep")
    W = g["W"]
    exact = {"plain": {}, "visc": dict(viscosity=0.05), "drag": dict(drag_rate=40.0)}
    for name, kw in exact.items():
        assert isothermal_timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, np.inf, 0.0, 1.0, **kw) == g[name], name
    assert isothermal_timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, np.inf, 0.999, 1.0) == g["clip"]
    assert isothermal_timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, 1e-4, 0.0, 1.0) == g["growth"]
    smag = isothermal_timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, np.inf, 0.0, 1.0, viscosity=1e-3,
                               smagorinsky_cs=2.0)
    assert_rel(smag, g["smag"], STEP_RTOL)


def test_smooth_problem_to_t02_matches_reference(golden):
    """The reference's CPU case: smooth 64x48, ppm4 + roe, rk3, cfl 0.4, t = 0.2."""
    from jathenax_gb300.run import evolve_isothermal
    g = golden("runs")
    U, time, dt, cycle = evolve_isothermal(g["smooth_U0"], 1 / 64, 1 / 48, 1.0, 1e-10, "rk3", 0.4,
                                           0.2, 100_000)
    assert cycle == g["smooth_cycle"]
    assert time == 0.2 and abs(time - g["smooth_time"]) <= 1e-15
    assert_rel(dt, g["smooth_dt"], RUN_RTOL)
    assert_rel(U, g["smooth_U"], RUN_RTOL)


def test_kh_wenoz_hlle_run_matches_reference(golden):
    from jathenax_gb300.run import evolve_isothermal
    g = golden("runs")
    U, time, _, cycle = evolve_isothermal(g["kh_U0"], 1 / 32, 1 / 32, 1.0, 1e-10, "rk3", 0.4, 0.1,
                                          100_000, reconstruct="wenoz", rsolver="hlle")
    assert cycle == g["kh_cycle"]
    assert_rel(U, g["kh_U"], RUN_RTOL)


def test_forced_turbulence_run_matches_reference(golden):
    from jathenax_gb300.forcing import cartesian_modes, forcing_basis
    from jathenax_gb300.run import evolve_isothermal
    g = golden("runs")
    x = (np.arange(32) + 0.5) / 32 - 0.5
    basis = forcing_basis(cartesian_modes(3, 5, (-5, 5), (-5, 5)), x, x, (1.0, 1.0))
    U, time, _, cycle = evolve_isothermal(
        g["turb_U0"], 1 / 32, 1 / 32, 1.0, 1.17549e-38, "rk3", 0.4, 0.5, 12, viscosity=1.5e-6,
        drag_rate=0.3333335, forcing=(g["turb_table"], basis), dt_update=0.0075, dedt=0.03703705)
    assert cycle == g["turb_cycle"] == 12
    assert_rel(time, g["turb_time"], RUN_RTOL)
    assert_rel(U, g["turb_U"], RUN_RTOL)


@pytest.mark.parametrize("shape", [(6, 6), (7, 5), (1, 9), (16, 33), (17, 64), (70, 37)])
def test_ragged_and_tiny_grids(G, shape):
    ny, nx = shape
    U0 = noisy_state(nx, ny, nvar=4, seed=ny * 100 + nx)
    for rec in ("ppm4", "wenoz", "dc"):
        gpu = G.isothermal_step(U0, 0.001, 1 / nx, 1 / ny, 1.0, 1e-10, "rk3", reconstruct=rec)
        ref = H.step(U0, 0.001, 1 / nx, 1 / ny, 1.0, 1e-10, "rk3", recon=rec)
        assert_rel(gpu, ref, STEP_RTOL, f"{shape} {rec}")


def test_density_floor_and_many_scalars(G):
    U0 = noisy_state(24, 20, nvar=9, seed=3)
    U0[3:6, 4:9, 0] = 1e-14  # below the floor: recovered as dfloor, momentum kept
    args = (1e-4, 1 / 24, 1 / 20, 1.0, 1e-10, "rk2")
    gpu = G.isothermal_step(U0, *args, reconstruct="ppmx", rsolver="llf")
    ref = H.step(U0, *args, recon="ppmx", solver="llf")
    assert_rel(gpu, ref, STEP_RTOL)


def test_explicit_tile_shapes_agree(G):
    import torch
    from jathenax_gb300 import _lib
    U0 = noisy_state(96, 80, nvar=4, seed=9)
    ref = H.step(U0, 0.001, 1 / 96, 1 / 80, 1.0, 1e-10, "rk3")
    for tile in ((8, 8), (16, 32), (64, 8), (32, 16), (128, 4)):
        desc = G.make_desc(U0.shape, torch.float64, 1 / 96, 1 / 80, 1.0, 1e-10, "rk3", tile=tile)
        ws, nbytes = _lib.workspace(desc)
        clock = _lib.new_clock(dt=0.001)
        Ud = _lib.to_device(U0)
        out, _ = G.run_stages(desc, Ud, clock=clock, ws=ws, nbytes=nbytes)
        assert_rel(out.cpu().numpy(), ref, STEP_RTOL, f"tile {tile}")


def test_float32_state_tracks_float64_oracle(G):
    U0 = noisy_state(64, 48, nvar=4, seed=21)
    ref = H.step(U0, 0.002, 1 / 64, 1 / 48, 1.0, 1e-10, "rk3")
    gpu = G.isothermal_step(U0.astype(np.float32), 0.002, 1 / 64, 1 / 48, 1.0, 1e-10, "rk3")
    assert gpu.dtype == np.float32
    assert max_rel_error(gpu, ref) < 1e-5


def test_face_operators_match_oracle():
    from jathenax_gb300 import fluxes as GF
    W = H.primitives(noisy_state(20, 14, nvar=4, seed=4), 1e-10)[1]
    for rec in RECONS:
        for axis in (0, 1):
            gl, gr = GF.reconstruct_faces(W, axis, rec, 1e-10)
            rl, rr = H.face_states(W, axis, rec, 1e-10)
            assert_rel(gl, rl, STEP_RTOL, f"{rec} left {axis}")
            assert_rel(gr, rr, STEP_RTOL, f"{rec} right {axis}")
            for rs in SOLVERS:
                assert_rel(GF.isothermal_flux(gl, gr, 1.0, axis, rs),
                           H.face_flux(rl, rr, 1.0, axis, rs), STEP_RTOL, f"{rec} {rs} {axis}")
    for axis in (0, 1):
        assert_rel(GF.viscous_momentum_flux(W, 1 / 20, 1 / 14, 1e-3, 0.2, axis),
                   H.viscous_flux(W, 1 / 20, 1 / 14, 1e-3, 0.2, axis), STEP_RTOL)
        gx, gy = GF.face_velocity_gradients(W, 1 / 20, 1 / 14, axis)
        rx, ry = H.face_gradients(W, 1 / 20, 1 / 14, axis)
        np.testing.assert_array_equal(gx, rx)
        np.testing.assert_array_equal(gy, ry)
        assert_rel(GF.smagorinsky_viscosity(gx, gy, 1 / 20, 1 / 14, 0.17)[..., None],
                   H.eddy_viscosity(rx, ry, 1 / 20, 1 / 14, 0.17)[..., None], STEP_RTOL)
    tau = noisy_state(20, 14, nvar=3, seed=8)
    for a, b in zip(GF.stress_face_fluxes(tau), H.sgs_face_flux(tau)):
        assert_rel(a, b, STEP_RTOL)
    fx, fy = noisy_state(20, 14, nvar=4, seed=1), noisy_state(20, 14, nvar=4, seed=2)
    assert_rel(GF.flux_divergence(fx, fy, 1 / 20, 1 / 14), H.divergence(fx, fy, 1 / 20, 1 / 14),
               STEP_RTOL)


def test_step_is_deterministic_and_conservative_at_1024(G):
    """Full-size property checks on the 1024^2 tanh Kelvin-Helmholtz state."""
    import torch
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    U0 = torch.as_tensor(kelvin_helmholtz_tanh(1024, 1024), device="cuda")
    a = G.isothermal_step(U0, 2e-4, 1 / 1024, 1 / 1024, 1.0, 1e-10, "rk3")
    b = G.isothermal_step(U0, 2e-4, 1 / 1024, 1 / 1024, 1.0, 1e-10, "rk3")
    assert torch.equal(a, b)
    before = U0.sum(dim=(0, 1))
    after = a.sum(dim=(0, 1))
    scale = U0.abs().sum(dim=(0, 1))
    assert torch.all((after - before).abs() <= 1e-13 * scale)


def tie_heavy_state(nx, ny, nvar, kind):
    """States full of exact ties, zeros and subnormal differences for the limiters.

    Densities are powers of two so that v = m / rho is recovered exactly and
    flat stencils stay exactly flat (otherwise rounding noise of 1e-17 sets
    the WENO-Z weights, whose epsilon is 1e-42, and the comparison measures
    noise amplification rather than the kernel).
    """
    x, y = R.cell_centers(nx, ny)
    X, Y = np.meshgrid(x, y)
    if kind == "steps":        # piecewise constant: flat stencils and jumps
        rho = np.where(np.abs(Y) < 0.25, 2.0, 1.0) * np.where(X > 0.1, 0.5, 1.0)
        vx = np.where(np.abs(Y) < 0.25, 0.5, -0.5)
        vy = np.zeros_like(X)
    elif kind == "linear":     # staircases: exact |dl| = |dh| ties
        rho = 2.0 ** np.round(X * 4)
        vx = 0.25 * np.round(Y * 16) / 16
        vy = -vx
    else:                      # subnormal-sized perturbations around exact values
        rho = 1.0 + np.where((np.arange(nx)[None, :] + np.arange(ny)[:, None]) % 3 == 0, 1e-300, 0.0)
        vx = np.where(X > 0, 5e-310, -5e-310) + 0.0 * Y
        vy = np.where(Y > 0, 0.0, -0.0) * X
    comps = [rho, rho * vx, rho * vy]
    for s in range(nvar - 3):
        comps.append(rho * np.where(X + s * 0.1 > 0, 1.0, 0.0))
    return np.stack(comps, axis=-1)


@pytest.mark.parametrize("kind", ["steps", "linear", "tiny"])
@pytest.mark.parametrize("rec", RECONS)
def test_limiters_on_ties_zeros_and_subnormals(G, kind, rec):
    U0 = tie_heavy_state(36, 20, 4, kind)
    for rs in SOLVERS:
        args = (1e-3, 1 / 36, 1 / 20, 1.0, 1e-10, "rk3")
        gpu = G.isothermal_step(U0, *args, reconstruct=rec, rsolver=rs)
        ref = H.step(U0, *args, recon=rec, solver=rs)
        assert_rel(gpu, ref, STEP_RTOL, f"{kind} {rec} {rs}")
        from jathenax_gb300 import fluxes as GF
        W = H.primitives(U0, 1e-10)[1]
        for axis in (0, 1):
            for a, b in zip(GF.reconstruct_faces(W, axis, rec, 1e-10), H.face_states(W, axis, rec, 1e-10)):
                assert_rel(a, b, STEP_RTOL, f"{kind} {rec} faces axis {axis}")


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_unaligned_state_pointers_use_the_generic_kernel(G, dtype):
    """4-variable states that are not 16-byte aligned take the scalar-access kernel."""
    import torch
    from jathenax_gb300 import _lib
    U0 = noisy_state(40, 24, nvar=4, seed=13)
    ref = H.step(U0, 0.001, 1 / 40, 1 / 24, 1.0, 1e-10, "rk3")
    tdtype = getattr(torch, dtype)
    n = U0.size
    # Views starting one element into larger buffers: 8- or 4-byte aligned only.
    bufs = [torch.zeros(n + 1, dtype=tdtype, device="cuda") for _ in range(3)]
    U_in, A, B = (b[1:].view(U0.shape) for b in bufs)
    U_in.copy_(torch.as_tensor(U0, device="cuda"))
    assert U_in.data_ptr() % 16 != 0
    desc = G.make_desc(U0.shape, tdtype, 1 / 40, 1 / 24, 1.0, 1e-10, "rk3")
    ws, nbytes = _lib.workspace(desc)
    clock = _lib.new_clock(dt=0.001)
    out, _ = G.run_stages(desc, U_in, clock=clock, ws=ws, nbytes=nbytes, out=A)
    tol = STEP_RTOL if dtype == "float64" else 1e-5
    assert_rel(out.cpu().numpy(), ref, tol)
