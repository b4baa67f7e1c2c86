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


def test_snapshot_vorticity_of_a_shear_and_a_rotation():
    from jathenax_gb300.diagnostics import snapshot_fields
    n = 64
    c = (np.arange(n) + 0.5) / n - 0.5
    X, Y = np.meshgrid(c, c)
    # vx = sin(2 pi y): vorticity -dvx/dy = -2 pi cos(2 pi y) * sin(2 pi h)/(2 pi h) (centred difference)
    U = np.stack((np.full((n, n), 2.0), 2.0 * np.sin(2 * np.pi * Y), np.zeros((n, n)), np.ones((n, n))), -1)
    f = snapshot_fields(U, 1 / n, 1 / n)
    h = 1 / n
    np.testing.assert_allclose(f["vorticity"], -np.cos(2 * np.pi * Y) * np.sin(2 * np.pi * h) / h, atol=1e-12)
    np.testing.assert_allclose(f["tracer"], 0.5)
    np.testing.assert_allclose(f["density"], 2.0)
    assert set(snapshot_fields(U[..., :3], h, h)) == {"density", "vorticity"}


def test_diagnostics_command_writes_spectra_csv_and_fields(tmp_path):
    from jathenax_gb300 import diagnostics
    n = 16
    c = (np.arange(n) + 0.5) / n - 0.5
    X, Y = np.meshgrid(c, c)
    U = np.stack((1 + 0.1 * np.sin(2 * np.pi * X), 0.3 * np.cos(2 * np.pi * Y), 0.2 * np.sin(2 * np.pi * X)), -1)
    np.savez(tmp_path / "run.npz", x=c, y=c, initial=U, conserved=U, time=0.0, dt=0.1, cycle=0)
    diagnostics.main([str(tmp_path / "run.npz")])
    table = np.loadtxt(tmp_path / "run_spectra.csv", delimiter=",", skiprows=1)
    modes, energy, enstrophy = diagnostics.shell_spectra(U)
    np.testing.assert_array_equal(table[:, 0], modes)
    np.testing.assert_allclose(table[:, 1], energy, rtol=1e-15)
    with np.load(tmp_path / "run_fields.npz") as f:
        assert {"final_density", "final_vorticity", "initial_vorticity"} <= set(f.files)


def test_shell_spectra_match_the_reference_script(golden):
    """The reference's own jathenax/spectra.py, run unmodified on these states
    (tests/golden/make_spectra.py), wrote the fixture's spectra; even, odd and
    unequal axes exercise the shell binning and the Nyquist derivative."""
    g = golden("spectra")
    names = sorted(k[:-2] for k in g if k.endswith("_U"))
    assert len(names) == 5
    for name in names:
        modes, energy, enstrophy = shell_spectra(g[f"{name}_U"])
        np.testing.assert_array_equal(modes, g[f"{name}_mode"], err_msg=name)
        np.testing.assert_allclose(energy, g[f"{name}_energy"], rtol=1e-14, atol=0, err_msg=name)
        np.testing.assert_allclose(enstrophy, g[f"{name}_enstrophy"], rtol=1e-14, atol=1e-300, err_msg=name)
