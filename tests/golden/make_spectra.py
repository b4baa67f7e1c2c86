"""Generate ``spectra.npz``: shell spectra computed by the reference's own analysis script.

Usage (needs the reference source tree, e.g. a checkout of JathenAX):

    python tests/golden/make_spectra.py --reference <path-to-JathenAX-checkout>

The reference's ``jathenax/spectra.py`` (kinetic energy of sqrt(rho) v and
enstrophy summed over integer shells floor(|k| + 0.5), the axis Nyquist
derivative dropped on even axes) is run unmodified as a script on snapshot
files of several states; matplotlib, which it imports for its figure, is
replaced by ``oracle/mplshim`` (plotting calls ignored). The script writes
its spectra as CSV with 17 significant digits, which round-trip float64
exactly; the fixture stores each input state and the CSV columns.
``tests/test_diagnostics.py`` checks ``jathenax_gb300.diagnostics.shell_spectra``
against them.
"""

import argparse
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
SHIM = REPO / "oracle" / "mplshim"


def states():
    """Random and structured states with even, odd and unequal axes."""
    rng = np.random.default_rng(2024)
    out = {}
    for ny, nx in ((24, 32), (25, 31), (32, 32), (17, 40)):
        rho = 1.0 + 0.4 * rng.random((ny, nx))
        v = 0.3 * rng.standard_normal((ny, nx, 2))
        out[f"random_{ny}x{nx}"] = np.concatenate((rho[..., None], rho[..., None] * v), axis=-1)
    n = 64
    x = (np.arange(n) + 0.5) / n - 0.5
    X, Y = np.meshgrid(x, x)
    inside = 0.5 * (np.tanh((Y + 0.25) / 0.01) - np.tanh((Y - 0.25) / 0.01))
    vy = 0.01 * np.sin(4 * np.pi * X) * (np.exp(-((Y - 0.25) / 0.05) ** 2) + np.exp(-((Y + 0.25) / 0.05) ** 2))
    out["kh_tanh_64"] = np.stack((np.ones_like(X), inside - 0.5, vy, inside), axis=-1)
    return out


def main():
    parser = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    parser.add_argument("--reference", type=Path, required=True)
    args = parser.parse_args()
    script = args.reference.resolve() / "jathenax" / "spectra.py"
    env = dict(os.environ, PYTHONPATH=str(SHIM), PYTHONDONTWRITEBYTECODE="1")
    fixture = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, U in states().items():
            snap = Path(tmp) / f"{name}.npz"
            np.savez(snap, conserved=U, time=np.float64(0.0))
            figure = Path(tmp) / f"{name}.png"
            run = subprocess.run([sys.executable, str(script), str(snap), "--output", str(figure)], env=env,
                                 cwd=tmp, capture_output=True, text=True)
            if run.returncode != 0:
                sys.exit(f"reference spectra.py failed on {name}:\n{run.stderr}")
            table = np.loadtxt(figure.with_suffix(".csv"), delimiter=",", skiprows=1)
            fixture[f"{name}_U"] = U
            fixture[f"{name}_mode"] = table[:, 0].astype(np.int64)
            fixture[f"{name}_energy"] = table[:, 1]
            fixture[f"{name}_enstrophy"] = table[:, 2]
            print(name, U.shape, "shells", len(table))
    np.savez_compressed(HERE / "spectra.npz", **fixture)
    print("wrote", HERE / "spectra.npz")


if __name__ == "__main__":
    main()
