"""The reference's own unit tests (tests/test_jathenax.py, tests/test_input.py of
JathenAX), restated against the GPU implementation with the same assertions
and tolerances.
"""

import subprocess
import sys
from math import factorial
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def jx():
    import jathenax_gb300.fluxes as fluxes
    import jathenax_gb300.forcing as forcing
    import jathenax_gb300.hydro as hydro
    import jathenax_gb300.initial_conditions as ic
    import jathenax_gb300.run as run
    return dict(fluxes=fluxes, forcing=forcing, hydro=hydro, ic=ic, run=run)


@pytest.mark.parametrize(("integrator", "order"), [("rk2", 2), ("rk3", 3), ("rk4", 4)])
def test_rk_stage_schedule(jx, integrator, order):
    # dU/dt = U: the schedule reproduces the Taylor polynomial (test_jathenax.py:23-36).
    hydro = jx["hydro"]
    dt = 0.125
    U = np.asarray(1.0)
    U_saved = U
    for coefficients in hydro.RK_STAGES[integrator]:
        U, U_saved = hydro.rk_stage(U, U_saved, -U, dt, coefficients)
    expected = sum(dt**n / factorial(n) for n in range(order + 1))
    np.testing.assert_allclose(U, expected, rtol=32 * np.finfo(np.float64).eps)


def test_rk3_zero_flux_preserves_float32_density(jx):
    hydro = jx["hydro"]
    rho = np.linspace(0.75, 1.25, 1024, dtype=np.float32)
    out = hydro.rk_stage(rho, rho, np.zeros_like(rho), 0.01, hydro.RK_STAGES["rk3"][-1])[0]
    np.testing.assert_array_equal(out, rho)


def test_density_floor_preserves_momentum(jx):
    U, W = jx["hydro"].recover_isothermal(np.asarray([[[0.125, 0.5, -0.25]]]), dfloor=0.25)
    np.testing.assert_array_equal(U, [[[0.25, 0.5, -0.25]]])
    np.testing.assert_array_equal(W, [[[0.25, 2.0, -1.0]]])


def test_isothermal_timestep_limits(jx):
    ts = jx["hydro"].isothermal_timestep
    W = np.asarray([[[1.0, 1.0, 2.0], [1.0, 3.0, 4.0]]])
    assert ts(W, 1.0, 2.0, 1.0, 0.5, np.inf, 0.0, 1.0) == 0.125
    assert ts(W, 1.0, 2.0, 1.0, 0.5, 0.03125, 0.0, 1.0) == 0.0625
    assert ts(W, 1.0, 2.0, 1.0, 0.5, np.inf, 0.9375, 1.0) == 0.0625


def test_viscous_timestep_limits(jx):
    ts = jx["hydro"].isothermal_timestep
    W = np.asarray([[[1.0, 0.0, 0.0]] * 2, [[1.0, 1.0, 0.0]] * 2])
    dx, dy, cfl = 0.25, 0.5, 0.5
    nu, Cs = 0.5, 2.0
    args = (dx, dy, 1.0, cfl, np.inf, 0.0, 1.0)
    assert ts(W, *args, viscosity=nu) == cfl * 0.25 * dx**2 / nu
    max_nu_sgs = Cs**2 * dx * dy / dy
    np.testing.assert_allclose(ts(W, *args, viscosity=nu, smagorinsky_cs=Cs),
                               cfl * (3 / 16) * dx**2 / (nu + 2 * max_nu_sgs))
    at_rest = W.copy()
    at_rest[..., 1] = 0.0
    assert ts(at_rest, *args, smagorinsky_cs=Cs) == cfl * dx


@pytest.mark.parametrize(("integrator", "order"), [("rk2", 2), ("rk3", 3), ("rk4", 4)])
def test_uniform_linear_drag(jx, integrator, order):
    hydro = jx["hydro"]
    initial = np.broadcast_to(np.asarray([2.0, 0.6, -0.4]), (6, 8, 3)).copy()
    dt, rate, cfl = 0.125, 4.0, 0.4
    _, W = hydro.recover_isothermal(initial, dfloor=1e-10)
    bound = hydro.isothermal_timestep(W, 1.0, 1.0, 1.0, cfl, np.inf, 0.0, 1.0, drag_rate=rate)
    np.testing.assert_allclose(bound, cfl / rate)
    final = hydro.isothermal_step(initial, dt, 1.0, 1.0, 1.0, 1e-10, integrator, drag_rate=rate)
    factor = sum((-rate * dt)**n / factorial(n) for n in range(order + 1))
    tol = 32 * np.finfo(np.float64).eps
    np.testing.assert_allclose(final[..., 0], initial[..., 0], rtol=tol)
    np.testing.assert_allclose(final[..., 1:], initial[..., 1:] * factor, rtol=tol)


def test_kick_normalization(jx):
    normalize_force = jx["forcing"].normalize_force
    rho = np.asarray([[[1.0], [2.0]]])
    raw_force = np.asarray([[[2.0, 1.0], [-1.0, 1.0]]])
    dt, dedt = 0.125, 0.04
    for sign in (-1.0, 1.0):
        momentum = sign * 0.125 * rho * raw_force
        U = np.concatenate((rho, momentum), axis=-1)
        force = normalize_force(U, raw_force, dt, dedt)
        delta = rho * force * dt
        energy = np.mean(0.5 * np.sum(delta * (2.0 * momentum + delta) / rho, axis=-1))
        tol = 64 * np.finfo(np.float64).eps
        np.testing.assert_allclose(delta.sum(axis=(0, 1)), 0.0, atol=tol)
        np.testing.assert_allclose(energy, dt * dedt, rtol=tol)
    np.testing.assert_array_equal(normalize_force(U, raw_force, dt, 0.0), 0.0)


@pytest.mark.parametrize("integrator", ["rk2", "rk3", "rk4"])
def test_periodic_step_conserves_mass_and_momentum(jx, integrator):
    nx, ny = 8, 6
    x, y = np.meshgrid(2.0 * np.pi * np.arange(nx) / nx, 2.0 * np.pi * np.arange(ny) / ny)
    rho = 1.0 + 0.2 * np.cos(x + y)
    U = np.stack((rho, 0.2 * rho * np.sin(y), 0.3 * rho * np.cos(x)), axis=-1)
    final = jx["hydro"].isothermal_step(U, 0.01, 1 / nx, 1 / ny, 1.0, 1e-10, integrator)
    assert np.max(np.abs(final - U)) > 1.0e-4
    np.testing.assert_allclose(final.mean(axis=(0, 1)), U.mean(axis=(0, 1)), rtol=0,
                               atol=16 * np.finfo(np.float64).eps)


@pytest.mark.parametrize("rsolver", ["llf", "hlle", "roe"])
def test_passive_scalars_share_mass_flux_without_changing_hydro(jx, rsolver):
    x = (np.arange(12) + 0.5) / 12 - 0.5
    U = jx["ic"].kelvin_helmholtz(x, x)
    np.testing.assert_array_equal(U[..., 0], 1.0)
    assert U[..., 3].min() == 0.0 and U[..., 3].max() == 1.0
    U = np.concatenate((U, 0.25 * U[..., :1]), axis=-1)
    force = np.broadcast_to(np.sin(2 * np.pi * x)[None, :, None], (12, 12, 2)).copy()

    def step(U):
        return jx["hydro"].isothermal_step(
            U, 0.01, 1 / 12, 1 / 12, 1.0, 1e-10, "rk3", viscosity=0.001, smagorinsky_cs=0.2,
            drag_rate=0.3, raw_force=force, dedt=0.04, rsolver=rsolver)

    final = step(U)
    tol = 32 * np.finfo(np.float64).eps
    np.testing.assert_allclose(final[..., :3], step(np.ascontiguousarray(U[..., :3])), rtol=0, atol=tol)
    np.testing.assert_allclose(final[..., 4], 0.25 * final[..., 0], rtol=0, atol=tol)
    np.testing.assert_allclose(final[..., 3:].mean(axis=(0, 1), dtype=np.float64), [0.5, 0.25],
                               rtol=0, atol=tol)
    assert np.max(np.abs(final[..., 3] - U[..., 3])) > 1e-4


def test_wenoz_float32_flat_stencils_at_jump(jx):
    W = np.asarray([[0.0, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 1.0]], dtype=np.float32)
    left, right = jx["fluxes"].wenoz_face_states(W, 1)
    np.testing.assert_allclose(left, np.roll(W, 1, axis=1), atol=2e-7)
    np.testing.assert_allclose(right, W, atol=2e-7)


def test_learned_stress_couples_conservatively(jx):
    fluxes = jx["fluxes"]
    nx, ny = 8, 5
    dx, dy = 1.0 / nx, 1.0 / ny
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dy
    k = 2.0 * np.pi
    vx, vy = np.meshgrid(np.sin(k * x), np.sin(k * y))
    w = [0.5, 2.0, -1.0, 1.5]
    dt = 0.125
    tau = np.stack((w[0] * vx, w[1] * vx + w[2] * vy, w[3] * vy), axis=-1)
    fx, fy = fluxes.stress_face_fluxes(tau)
    result = -dt * fluxes.flux_divergence(fx, fy, dx, dy)
    dvx_dx = np.cos(k * x)[None, :] * np.sin(k * dx) / dx
    dvy_dy = np.cos(k * y)[:, None] * np.sin(k * dy) / dy
    expected = -dt * np.stack((0.5 * dvx_dx - dvy_dy, 2.0 * dvx_dx + 1.5 * dvy_dy), axis=-1)
    tol = 32 * np.finfo(np.float64).eps
    np.testing.assert_allclose(result, expected, rtol=tol, atol=tol)
    np.testing.assert_allclose(result.sum(axis=(0, 1)), 0.0, atol=tol * nx * ny)


@pytest.mark.parametrize("integrator", ["rk2", "rk3", "rk4"])
def test_sgs_predictor_uses_each_stage_and_conserves_momentum(jx, integrator):
    import torch
    hydro, fluxes = jx["hydro"], jx["fluxes"]
    x = (np.arange(8) + 0.5) / 8 - 0.5
    U = jx["ic"].kelvin_helmholtz(x, x)
    scale = torch.tensor([0.0125, 0.025, -0.0375], dtype=torch.float64, device="cuda")

    def predict_stress(weights, W):
        assert W.shape == (8, 8, 3)
        return weights["scale"] * W

    def step(weights):
        return hydro.isothermal_step(U, 0.01, 1 / 8, 1 / 8, 1.0, 1e-10, integrator, trace=True,
                                     predict_stress=predict_stress, sgs_weights=weights)

    final, stages = step({"scale": scale})
    baseline, _ = step({"scale": torch.zeros_like(scale)})
    assert np.max(np.abs(final[..., 1:3] - baseline[..., 1:3])) > 1e-4
    tol = 16 * np.finfo(np.float64).eps
    for stage in stages:
        tau = scale.cpu().numpy() * stage["primitives"][..., :3]
        for axis, d, comps in ((1, "x", slice(0, 2)), (0, "y", slice(1, 3))):
            gas = fluxes.isothermal_flux(stage[f"left_{d}"], stage[f"right_{d}"], 1.0, axis)
            stress = tau[..., comps]
            expected = 0.5 * (stress + np.roll(stress, 1, axis=axis))
            added = stage[f"flux_{d}"] - gas
            np.testing.assert_allclose(added[..., 1:3], expected, rtol=0, atol=tol)
            np.testing.assert_allclose(added[..., [0, 3]], 0.0, rtol=0, atol=tol)
    np.testing.assert_allclose(final.mean(axis=(0, 1)), U.mean(axis=(0, 1)), rtol=0, atol=tol)


def test_zero_sgs_predictor_matches_baseline_evolution(jx):
    import torch
    x = (np.arange(8) + 0.5) / 8 - 0.5
    U = jx["ic"].kelvin_helmholtz(x, x)
    args = (U, 1 / 8, 1 / 8, 1.0, 1e-10, "rk3", 0.4, 0.1, 10)
    evolve = jx["run"].evolve_isothermal
    baseline = evolve(*args)
    coupled = evolve(*args, predict_stress=lambda w, W: torch.zeros_like(W))
    for a, b in zip(baseline, coupled, strict=True):
        np.testing.assert_array_equal(a, b)


def test_sgs_predictor_requires_the_full_grid(jx):
    U = np.ones((6, 8, 3))
    with pytest.raises(ValueError, match="predict_stress must return"):
        jx["hydro"].isothermal_step(U, 0.01, 1 / 8, 1 / 6, 1.0, 1e-10, "rk3",
                                    predict_stress=lambda weights, W: W[:1])


def test_input_deck_and_cli_overrides(tmp_path):
    deck = tmp_path / "input.toml"
    deck.write_text("""
[problem]
name = "kh"

[mesh]
nx = 8
ny = 10

[time]
nlim = 2
tlim = 1
integrator = "rk2"

[hydro]
reconstruct = "plm"
rsolver = "hlle"

[output]
file = "configured.npz"
""")
    output = tmp_path / "overridden.npz"
    env = {"PYTHONPATH": str(REPO)}
    import os
    env = dict(os.environ, **env)
    result = subprocess.run(
        [sys.executable, "-m", "jathenax_gb300.run", "-i", str(deck), "--nx", "12",
         "--integrator", "rk4", "--rsolver", "llf", "--output", str(output)],
        cwd=tmp_path, capture_output=True, text=True, env=env)
    assert result.returncode == 0, result.stderr
    assert "RK4" in result.stdout
    assert "Reconstruction plm, Riemann solver llf" in result.stdout
    with np.load(output) as data:
        assert data["problem"].item() == "kh"
        assert data["conserved"].shape == (10, 12, 4)
        assert data["cycle"] == 2
        assert 0 < data["time"] < 1
    assert not (tmp_path / "configured.npz").exists()
