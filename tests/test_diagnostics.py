"""Spectrum and error diagnostics (host NumPy; no GPU)."""

import numpy as np

from jathenax_gb300.diagnostics import precision_report, relative_l1, shell_spectra


def test_shell_energy_sums_to_the_kinetic_energy():
    # The reference's own self-check (spectra.py:42): Parseval over all shells.
    rng = np.random.default_rng(0)
    ny, nx = 24, 32
    rho = 1.0 + 0.3 * rng.random((ny, nx))
    v = rng.standard_normal((ny, nx, 2))
    U = np.concatenate((rho[..., None], rho[..., None] * v), axis=-1)
    _, energy, enstrophy = shell_spectra(U)
    np.testing.assert_allclose(energy.sum(), 0.5 * np.mean(rho * (v**2).sum(-1)), rtol=1e-12)
    assert np.all(enstrophy >= 0)


def test_single_mode_lands_in_its_shell():
    n = 32
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    U = np.zeros((n, n, 3))
    U[..., 0] = 1.0
    U[..., 2] = np.sin(2 * np.pi * 5 * X)  # vy(x): kx = +-5
    modes, energy, enstrophy = shell_spectra(U)
    assert np.argmax(energy) == 5 and energy[5] > 0.99 * energy.sum()
    # |omega|^2 = (2 pi k)^2 |v|^2 for one mode
    np.testing.assert_allclose(enstrophy[5], (2 * np.pi * 5)**2 * energy[5], rtol=1e-12)


def test_precision_report_is_zero_for_identical_states():
    rng = np.random.default_rng(1)
    U = np.concatenate((1 + rng.random((16, 16, 1)), rng.standard_normal((16, 16, 2))), axis=-1)
    rep = precision_report(U, U, U, 1 / 16, 1 / 16)
    assert rep["l1_density"] == 0 and rep["l1_momentum"] == 0 and rep["ke_spectrum_max_rel_dev"] == 0
    np.testing.assert_array_equal(relative_l1(U + 1e-3, U)[0] > 0, True)
