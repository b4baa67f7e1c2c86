"""The reference's analytic viscosity checks on a periodic sinusoidal shear
(validation/periodic_shear.py), run on the GPU in float64.

A 256² unit square at rest density 1 carries vy = 0.5 sin(16 pi x). With
uniform viscosity the shear decays at the rate of the centred discrete
Laplacian, so the kinetic energy at t = 5 is E0 exp(-2 nu k_h^2 t) with
k_h^2 = 4 sin^2(k h / 2) / h^2; with Smagorinsky viscosity the first step's
fractional energy loss rate is (16 / 3 pi) (Cs h)^2 A k^3, the continuum mean
of |cos|^3 being 4 / (3 pi). Density and vx stay exactly uniform / zero to
the validation's 2e-11, and the diffusion limits set dt to 5e-13.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, MODE, AMPLITUDE = 256, 8, 0.5
H, CS, CFL, TLIM = 1.0 / N, 1.0, 0.4, 5.0
K = 2.0 * np.pi * MODE


def shear_state():
    x = (np.arange(N) + 0.5) * H
    U = np.zeros((N, N, 3))
    U[..., 0] = 1.0
    U[..., 2] = AMPLITUDE * np.sin(K * x)
    return U


def kinetic_energy(U):
    return 0.5 * np.mean(np.sum(U[..., 1:] ** 2, axis=-1) / U[..., 0])


def evolve(U, nlim, tlim=TLIM, **kw):
    from jathenax_gb300.run import evolve_isothermal
    return evolve_isothermal(U, H, H, CS, 1e-10, "rk3", CFL, tlim, nlim, **kw)


def test_uniform_viscosity_decays_at_the_discrete_laplacian_rate():
    nu = 1.5e-5
    U = shear_state()
    final, time, _, cycles = evolve(U, 10_000, viscosity=nu)
    assert time == TLIM and 0 < cycles < 10_000
    np.testing.assert_allclose(final[..., 0], 1.0, rtol=0, atol=2e-11)
    np.testing.assert_allclose(final[..., 1], 0.0, rtol=0, atol=2e-11)
    assert abs(final[..., 2].mean()) <= 2e-11
    k_grid_sq = 4.0 * np.sin(K * H / 2.0) ** 2 / H ** 2
    expected = kinetic_energy(U) * np.exp(-2.0 * nu * k_grid_sq * TLIM)
    np.testing.assert_allclose(kinetic_energy(final), expected, rtol=2e-9)


def test_smagorinsky_run_and_initial_loss_rate():
    cs_smag = 0.2
    U = shear_state()
    E0 = kinetic_energy(U)
    final, time, _, _ = evolve(U, 10_000, smagorinsky_cs=cs_smag)
    assert time == TLIM
    np.testing.assert_allclose(final[..., 0], 1.0, rtol=0, atol=2e-11)
    np.testing.assert_allclose(final[..., 1], 0.0, rtol=0, atol=2e-11)
    assert abs(final[..., 2].mean()) <= 2e-11
    first, _, first_dt, cycles = evolve(U, 1, smagorinsky_cs=cs_smag)
    assert cycles == 1
    loss_rate = (E0 - kinetic_energy(first)) / (first_dt * E0)
    exact = 16.0 / (3.0 * np.pi) * (cs_smag * H) ** 2 * AMPLITUDE * K ** 3
    np.testing.assert_allclose(loss_rate, exact, rtol=0.01)


@pytest.mark.parametrize("nu,cs_smag", [(0.01, 0.0), (0.0, 8.0)])
def test_diffusion_limits_set_the_timestep(nu, cs_smag):
    from jathenax_gb300.hydro import isothermal_timestep
    U = shear_state()
    dt = float(isothermal_timestep(U, H, H, CS, CFL, np.inf, 0.0, TLIM, viscosity=nu,
                                   smagorinsky_cs=cs_smag))
    if cs_smag > 0.0:
        max_face_strain = 2.0 * AMPLITUDE * np.sin(K * H / 2.0) / H
        nu_max = (cs_smag * H) ** 2 * max_face_strain
        expected = CFL * (3.0 / 16.0) * H ** 2 / (2.0 * nu_max)
    else:
        expected = CFL * 0.25 * H ** 2 / nu
    np.testing.assert_allclose(dt, expected, rtol=5e-13)
    _, _, _, cycles = evolve(U, 2, viscosity=nu, smagorinsky_cs=cs_smag)
    assert cycles == 2
