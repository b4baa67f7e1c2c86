"""Diagnostics on host copies of states: spectra, fields, errors, drift.

``shell_spectra`` restates the reference's analysis script
(jathenax/spectra.py:22-41): density-weighted kinetic energy of sqrt(rho) v
and the Fourier-curl enstrophy, summed over integer shells
floor(|k| + 0.5). ``snapshot_fields`` restates the fields of
jathenax/plot_snapshot.py:25-33 (tracer concentration, density and the
centred-difference vorticity). Neither plots (matplotlib is not a
dependency): ``python -m jathenax_gb300.diagnostics snapshot.npz`` writes the
spectra CSV of spectra.py (``mode,kinetic_energy,enstrophy``) and the fields
as an npz instead of figures. The error helpers are the Precision pattern's
metrics: relative L1 error per component, box-integrated drift of the
conserved sums (run.py:186-187), and the kinetic-energy spectrum deviation.
"""

import argparse
from pathlib import Path

import numpy as np


def shell_spectra(U):
    """Return (modes, kinetic_energy, enstrophy) per integer shell (spectra.py:22-41)."""
    U = np.asarray(U, dtype=np.float64)
    rho, mx, my = np.moveaxis(U[..., :3], -1, 0)
    ny, nx = rho.shape
    kx, ky = np.fft.fftfreq(nx) * nx, np.fft.fftfreq(ny) * ny
    radius = np.hypot(kx[None, :], ky[:, None])
    shell = np.floor(radius + 0.5).astype(int)
    modes = np.arange(shell.max() + 1)
    vx, vy = mx / rho, my / rho
    root = np.sqrt(rho)
    ax = np.fft.fft2(root * vx) / rho.size
    ay = np.fft.fft2(root * vy) / rho.size
    energy = np.bincount(shell.ravel(), (0.5 * (np.abs(ax)**2 + np.abs(ay)**2)).ravel(),
                         minlength=len(modes))
    # The axis Nyquist mode has no real derivative.
    kxd, kyd = kx.copy(), ky.copy()
    if nx % 2 == 0:
        kxd[nx // 2] = 0
    if ny % 2 == 0:
        kyd[ny // 2] = 0
    omega = 2j * np.pi * (kxd[None, :] * np.fft.fft2(vy) - kyd[:, None] * np.fft.fft2(vx))
    enstrophy = np.bincount(shell.ravel(), (0.5 * np.abs(omega / rho.size)**2).ravel(),
                            minlength=len(modes))
    return modes, energy, enstrophy


def snapshot_fields(U, dx, dy):
    """{"tracer" (4+ variables), "density", "vorticity"} of a state (plot_snapshot.py:25-33).

    Vorticity is dvy/dx - dvx/dy by periodic centred differences.
    """
    U = np.asarray(U, dtype=np.float64)
    rho, mx, my = np.moveaxis(U[..., :3], -1, 0)
    vx, vy = mx / rho, my / rho
    dvy_dx = (np.roll(vy, -1, axis=1) - np.roll(vy, 1, axis=1)) / (2 * dx)
    dvx_dy = (np.roll(vx, -1, axis=0) - np.roll(vx, 1, axis=0)) / (2 * dy)
    fields = {"density": rho, "vorticity": dvy_dx - dvx_dy}
    if U.shape[-1] > 3:
        fields["tracer"] = U[..., 3] / rho
    return fields


def relative_l1(a, b):
    """Per component: mean |a - b| / mean |b| over the grid (float64)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    num = np.mean(np.abs(a - b), axis=(0, 1))
    den = np.maximum(np.mean(np.abs(b), axis=(0, 1)), 1e-300)
    return num / den


def box_drift(U, U0, dx, dy):
    """Change of the box-integrated conserved quantities (run.py:186-187)."""
    return (np.asarray(U).sum(axis=(0, 1), dtype=np.float64)
            - np.asarray(U0).sum(axis=(0, 1), dtype=np.float64)) * dx * dy


def spectrum_deviation(U, U_ref, shells=None, spectra=None):
    """Largest relative deviation of the KE shell spectrum over shells
    1..shells-1 (default min(nx, ny)//2 - 1). `spectra` = precomputed
    (energy, energy_ref)."""
    e, e_ref = spectra if spectra is not None else (shell_spectra(U)[1], shell_spectra(U_ref)[1])
    ny, nx = np.shape(U)[:2]
    hi = shells if shells is not None else max(2, min(nx, ny) // 2)
    sl = slice(1, hi)
    ref = np.maximum(e_ref[sl], 1e-300)
    return float(np.max(np.abs(e[sl] - e_ref[sl]) / ref))


def precision_report(U32, U64, U0, dx, dy):
    """The FP32-vs-FP64 error record used by the Precision pattern. The
    spectrum deviation is given over all shells and over shells below 64
    (where the energy is; near the grid scale the shells hold so little
    energy that any difference is a large relative one)."""
    l1 = relative_l1(U32, U64)
    drift32 = box_drift(U32, U0, dx, dy)
    drift64 = box_drift(U64, U0, dx, dy)
    spectra = (shell_spectra(U32)[1], shell_spectra(U64)[1])
    return {
        "l1_density": float(l1[0]),
        "l1_momentum": float(max(l1[1], l1[2])),
        "drift_fp32": [float(v) for v in drift32[:3]],
        "drift_fp64": [float(v) for v in drift64[:3]],
        "ke_spectrum_max_rel_dev": spectrum_deviation(U32, U64, spectra=spectra),
        "ke_spectrum_max_rel_dev_k<64": spectrum_deviation(U32, U64, shells=min(64, max(2, min(np.shape(U64)[:2]) // 2)),
                                                           spectra=spectra),
    }


def main(argv=None):
    parser = argparse.ArgumentParser(description="Spectra and fields of a run's npz output (no plots).")
    parser.add_argument("snapshot", type=Path, help="npz written by jathenax_gb300.run")
    parser.add_argument("--output", type=Path, help="Output stem (default: next to the snapshot)")
    args = parser.parse_args(argv)
    stem = args.output or args.snapshot.with_suffix("")
    with np.load(args.snapshot) as snap:
        x, y = snap["x"], snap["y"]
        initial, final = (snap[key].astype(np.float64) for key in ("initial", "conserved"))
    dx, dy = float(x[1] - x[0]), float(y[1] - y[0])
    modes, energy, enstrophy = shell_spectra(final)
    spectra = Path(f"{stem}_spectra.csv")
    spectra.parent.mkdir(parents=True, exist_ok=True)
    np.savetxt(spectra, np.column_stack((modes, energy, enstrophy)), delimiter=",",
               header="mode,kinetic_energy,enstrophy", comments="", fmt=("%d", "%.16e", "%.16e"))
    fields = Path(f"{stem}_fields.npz")
    arrays = {f"{when}_{name}": value for when, U in (("initial", initial), ("final", final))
              for name, value in snapshot_fields(U, dx, dy).items()}
    np.savez(fields, x=x, y=y, **arrays)
    print(spectra)
    print(fields)


if __name__ == "__main__":
    main()
