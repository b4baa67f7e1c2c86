"""The command line (drop-in for ``python -m jathenax.run``) on the GPU: the
reference's flags, an SGS model module loaded by name with its weights file,
the npz output keys, and checkpoint/resume from the command line."""

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

# The reference's example SGS predictor (a constant eddy viscosity), written
# for the hook's torch CUDA tensors.
SGS_MODULE = '''
import numpy as np
import torch


def load_weights(checkpoint):
    if checkpoint is None:
        return {"nu": 1e-3}
    with np.load(checkpoint, allow_pickle=False) as saved:
        return {"nu": float(saved["nu"])}


def predict_stress(weights, primitives):
    ny, nx, _ = primitives.shape
    rho, v = primitives[..., 0], primitives[..., 1:3]
    dv_dx = (torch.roll(v, -1, 1) - torch.roll(v, 1, 1)) * (0.5 * nx)
    dv_dy = (torch.roll(v, -1, 0) - torch.roll(v, 1, 0)) * (0.5 * ny)
    dvx_dx, dvy_dy = dv_dx[..., 0], dv_dy[..., 1]
    shear = dv_dx[..., 1] + dv_dy[..., 0]
    trace = (2.0 / 3.0) * (dvx_dx + dvy_dy)
    strain = torch.stack((2.0 * dvx_dx - trace, shear, 2.0 * dvy_dy - trace), dim=-1)
    return -(rho * weights["nu"])[..., None] * strain
'''


def run_cli(tmp_path, *args):
    env = dict(os.environ, PYTHONPATH=f"{tmp_path}{os.pathsep}{ROOT}")
    result = subprocess.run([sys.executable, "-m", "jathenax_gb300.run", *map(str, args)], cwd=ROOT, env=env,
                            capture_output=True, text=True, timeout=600)
    assert result.returncode == 0, result.stderr[-2000:]
    return result.stdout


def test_cli_runs_an_sgs_model_with_weights(tmp_path):
    (tmp_path / "toy_sgs.py").write_text(SGS_MODULE)
    np.savez(tmp_path / "weights.npz", nu=np.float64(2e-3))
    out = tmp_path / "kh.npz"
    run_cli(tmp_path, "kh", "--nx", 32, "--ny", 24, "--tlim", 0.02, "--sgs-model", "toy_sgs", "--sgs-weights",
            tmp_path / "weights.npz", "--output", out)
    with np.load(out) as saved:
        assert {"x", "y", "initial", "conserved", "time", "dt", "cycle", "problem", "sgs_model"} <= set(saved.files)
        assert str(saved["sgs_model"]) == "toy_sgs" and float(saved["time"]) == 0.02
        final = saved["conserved"]
    # The same run in-process, through evolve_isothermal with the hook.
    sys.path.insert(0, str(tmp_path))
    try:
        import toy_sgs
        from jathenax_gb300.initial_conditions import cell_centers, kelvin_helmholtz
        from jathenax_gb300.run import evolve_isothermal
        x, y = cell_centers(32, 24)
        U0 = kelvin_helmholtz(x, y)
        U, t, _, _ = evolve_isothermal(U0, 1 / 32, 1 / 24, 1.0, 1e-10, "rk3", 0.4, 0.02, 100000,
                                       predict_stress=toy_sgs.predict_stress,
                                       sgs_weights=toy_sgs.load_weights(tmp_path / "weights.npz"))
    finally:
        sys.path.remove(str(tmp_path))
    np.testing.assert_array_equal(final, U)


def test_cli_checkpoint_then_resume_matches_one_run(tmp_path):
    deck = tmp_path / "smooth.toml"
    deck.write_text('[problem]\nname = "smooth"\n[mesh]\nnx = 40\nny = 32\n[time]\ntlim = 10.0\nnlim = 30\n')
    run_cli(tmp_path, "-i", deck, "--output", tmp_path / "full.npz")
    short = tmp_path / "short.toml"
    short.write_text('[problem]\nname = "smooth"\n[mesh]\nnx = 40\nny = 32\n[time]\ntlim = 10.0\nnlim = 12\n')
    run_cli(tmp_path, "-i", short, "--output", tmp_path / "part.npz", "--checkpoint", tmp_path / "ck.npz")
    run_cli(tmp_path, "-i", deck, "--output", tmp_path / "resumed.npz", "--resume", tmp_path / "ck.npz")
    with np.load(tmp_path / "full.npz") as a, np.load(tmp_path / "resumed.npz") as b:
        assert int(a["cycle"]) == int(b["cycle"]) == 30 and float(a["time"]) == float(b["time"])
        np.testing.assert_array_equal(a["conserved"], b["conserved"])
