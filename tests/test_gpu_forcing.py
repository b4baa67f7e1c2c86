"""The forcing kernels on shapes the golden fixtures do not reach: the tiled
render on ragged grids (sides not multiples of the 32x32 render tile), mode
counts that are not a multiple of the 8-mode chunk, the NaN field of an
update past the table, and the float32 normalisation sums (TwoSum pairs)
against the float64 oracle (forcing.py:103-149)."""

import numpy as np
import pytest
from conftest import STEP_RTOL, assert_rel, max_rel_error

from oracle import forcing_oracle as F
from oracle import hydro_oracle as H
from oracle import run_oracle as R

pytestmark = pytest.mark.gpu

# Float32 tolerances against the float64 oracle, relative to the largest
# magnitude: the render adds 4 float32 FMAs per mode (56 modes) and the sums
# run over up to 10^4 cells.
F32_RENDER_RTOL = 2e-6
F32_ACCEL_RTOL = 1e-5


def amplitudes(n_modes, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n_modes, 2, 2))


def modes_subset(n_modes, seed):
    full = F.forcing_modes(3, 5, (-5, 5), (-5, 5))
    if n_modes <= len(full):
        return full[:n_modes]
    rng = np.random.default_rng(seed)
    return rng.integers(-7, 8, size=(n_modes, 2))


@pytest.mark.parametrize("nx,ny", [(45, 37), (96, 64), (33, 130), (1, 5)])
@pytest.mark.parametrize("n_modes", [56, 13, 1])
def test_render_matches_oracle_on_ragged_grids(nx, ny, n_modes):
    from jathenax_gb300 import forcing as GF
    modes = modes_subset(n_modes, nx + ny)
    x, y = R.cell_centers(nx, ny)
    amp = amplitudes(n_modes, n_modes)
    ref = F.render(amp, F.phase_tables(modes, x, y, (1.0, 1.0)))
    basis = GF.forcing_basis(modes, x, y, (1.0, 1.0))
    got = GF.render_force(amp, basis).cpu().numpy()
    assert got.shape == (ny, nx, 2)
    assert_rel(got, ref, STEP_RTOL, "float64 render")
    import torch
    got32 = GF.render_force(amp, basis, dtype=torch.float32).cpu().numpy()
    assert got32.dtype == np.float32
    assert max_rel_error(got32, ref) <= F32_RENDER_RTOL


def test_update_past_the_table_renders_nan():
    from jathenax_gb300 import forcing as GF
    modes = F.forcing_modes(3, 5, (-5, 5), (-5, 5))
    x, y = R.cell_centers(40, 24)
    basis = GF.forcing_basis(modes, x, y, (1.0, 1.0))
    table = np.stack([amplitudes(len(modes), s) for s in range(3)])
    update, raw = GF.update_force(0.1, 2, np.zeros((24, 40, 2)), table, basis, 0.03, 0.0)
    raw = raw.cpu().numpy()
    assert int(update) == 3 and raw.shape == (24, 40, 2) and np.all(np.isnan(raw))
    update, raw = GF.update_force(0.07, 1, np.zeros((24, 40, 2)), table, basis, 0.03, 0.0)
    raw = raw.cpu().numpy()
    ref = F.render(table[2], F.phase_tables(modes, x, y, (1.0, 1.0)))
    assert int(update) == 2
    assert_rel(raw, ref, STEP_RTOL, "in-table render")


@pytest.mark.parametrize("nx,ny", [(64, 48), (130, 77)])
def test_float32_normalisation_sums_match_float64_oracle(nx, ny):
    import torch
    from jathenax_gb300 import forcing as GF
    rng = np.random.default_rng(nx)
    x, y = R.cell_centers(nx, ny)
    X, Y = np.meshgrid(x, y)
    rho = 1.0 + 0.3 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y) + 0.05 * rng.random((ny, nx))
    U = np.stack((rho, rho * 0.2 * np.sin(2 * np.pi * Y), rho * 0.1 * np.cos(2 * np.pi * X)), axis=-1)
    modes = F.forcing_modes(3, 5, (-5, 5), (-5, 5))
    raw = F.render(amplitudes(len(modes), 7), F.phase_tables(modes, x, y, (1.0, 1.0)))
    U32, raw32 = U.astype(np.float32), raw.astype(np.float32)
    ref = H.normalized_acceleration(U32.astype(np.float64), raw32.astype(np.float64), 0.003, 0.04)
    got = GF.normalize_force(torch.as_tensor(U32, device="cuda"), torch.as_tensor(raw32, device="cuda"),
                             0.003, 0.04).cpu().numpy()
    assert got.dtype == np.float32
    assert max_rel_error(got, ref) <= F32_ACCEL_RTOL
    assert_rel(GF.normalize_force(U, raw, 0.003, 0.04), H.normalized_acceleration(U, raw, 0.003, 0.04),
               STEP_RTOL, "float64 normalisation")
