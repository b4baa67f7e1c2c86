"""Batches of uneven solves: each result is bitwise the same alone and in the mix."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_solve(kind, n, dtype, recon, rsolver, integrator, tlim, tile_y, clock=None, seed=1618, tile_x=32):
    import torch
    from jathenax_gb300.forcing import cartesian_modes, forcing_basis, modal_coefficients
    from jathenax_gb300.initial_conditions import (
        cell_centers, kelvin_helmholtz_tanh, smooth_waves, uniform_rest)
    from jathenax_gb300.solver import Solve
    tdtype = getattr(torch, dtype)
    kw = dict(reconstruct=recon, rsolver=rsolver, tile=(tile_x, tile_y), dtype=tdtype, clock=clock)
    if kind == "kh":
        U = kelvin_helmholtz_tanh(n, n)
        return Solve(U, 1 / n, 1 / n, 1.0, 1e-10, integrator, 0.4, tlim, 10**6, **kw)
    if kind == "smooth":
        return Solve(smooth_waves(n, n + 8), 1 / n, 1 / (n + 8), 1.0, 1e-10, integrator, 0.4, tlim,
                     10**6, **kw)
    x, _ = cell_centers(n, n)
    modes = cartesian_modes(3, 5, (-5, 5), (-5, 5))
    updates = int(np.ceil(tlim / 0.0075)) + 1
    table = modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, seed, 0.75, 0.0075, updates)
    basis = forcing_basis(modes, x, x, (1.0, 1.0))
    return Solve(uniform_rest(n, n), 1 / n, 1 / n, 1.0, 1.17549e-38, integrator, 0.4, tlim, 10**6,
                 viscosity=1.5e-6, drag_rate=0.3333335, forcing=(table, basis), dt_update=0.0075,
                 dedt=0.03703705, **kw)


SPECS = [  # kind, n, dtype, recon, rsolver, integrator, tlim
    ("kh", 64, "float32", "ppm4", "roe", "rk3", 0.05),
    ("kh", 96, "float32", "ppm4", "roe", "rk3", 0.03),
    ("turb", 48, "float32", "ppm4", "roe", "rk3", 0.06),
    ("turb", 32, "float32", "ppm4", "roe", "rk3", 0.04),
    ("smooth", 40, "float64", "wenoz", "hlle", "rk4", 0.02),
    ("kh", 72, "float64", "ppmx", "llf", "rk2", 0.03),
    ("smooth", 24, "float32", "plm", "roe", "rk3", 0.05),
]


def run_alone(spec, tile_y, tile_x=32):
    s = make_solve(*spec, tile_y=tile_y, tile_x=tile_x)
    s.run(steps_per_sync=8)
    c = s.state()
    return s.S.cpu().numpy(), c.time, c.cycle


@pytest.mark.parametrize("tile", [(32, 16), (58, 16), (0, 0)])
def test_batch_results_equal_solo_results_bitwise(tile):
    from jathenax_gb300.batch import Batch, ClockBank
    tile_x, tile_y = tile
    bank = ClockBank(len(SPECS))
    solves = [make_solve(*spec, tile_y=tile_y, tile_x=tile_x, clock=bank.slot(i)) for i, spec in enumerate(SPECS)]
    batch = Batch(solves, clocks=bank)
    # 4 (precision, method) classes; marching groups split by variable count
    assert batch.groups == {(32, 16): 4, (58, 16): 5, (0, 0): 5}[tile]
    clocks = batch.run(steps_per_sync=8)
    for spec, s, c in zip(SPECS, solves, clocks):
        U_alone, t_alone, cyc_alone = run_alone(spec, tile_y, tile_x)
        assert c.done and c.cycle == cyc_alone and c.time == t_alone, spec
        np.testing.assert_array_equal(s.S.cpu().numpy(), U_alone, err_msg=str(spec))


@pytest.mark.parametrize("tile_x", [32, 58])
def test_batch_tile_height_does_not_change_results(tile_x):
    from jathenax_gb300.batch import Batch
    outs = []
    for tile_y in (8, 32):
        solves = [make_solve(*spec, tile_y=tile_y, tile_x=tile_x) for spec in SPECS[:4]]
        Batch(solves, blocks_per_sm=2).run(steps_per_sync=4, use_graph=False)
        outs.append([s.S.cpu().numpy() for s in solves])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


def test_batch_mixes_tiles_and_kernels_bitwise():
    """Solves of one group with different tiles, and both kernels side by side."""
    from jathenax_gb300.batch import Batch
    tiles = [(32, 16), (32, 8), (58, 8), (58, 32), (0, 0), (32, 32), (58, 64)]
    solves = [make_solve(*spec, tile_y=ty, tile_x=tx) for spec, (tx, ty) in zip(SPECS, tiles)]
    batch = Batch(solves)
    # The float32 ppm4/roe class runs both kernels, its 3-variable marching
    # solves in two groups (8 rows: register path; 32 rows: the row ring).
    assert batch.groups == 6
    batch.run(steps_per_sync=4)
    for spec, s, (tx, ty) in zip(SPECS, solves, tiles):
        U_alone, _, _ = run_alone(spec, ty, tx)
        np.testing.assert_array_equal(s.S.cpu().numpy(), U_alone, err_msg=f"{spec} {tx}x{ty}")


def test_batch_rejects_other_tiles_and_wide_states():
    from jathenax_gb300.batch import Batch
    import torch
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    from jathenax_gb300.solver import Solve
    a = make_solve("kh", 32, "float32", "ppm4", "roe", "rk3", 0.01, tile_y=16, tile_x=16)
    with pytest.raises(ValueError, match="batch tiles"):
        Batch([a])
    U = kelvin_helmholtz_tanh(32, 32)
    wide = Solve(np.concatenate([U, U[..., 3:]], axis=-1), 1 / 32, 1 / 32, 1.0, 1e-10, "rk3", 0.4, 0.01, 10,
                 dtype=torch.float32)
    with pytest.raises(ValueError, match="3 or 4 variables"):
        Batch([wide])


def test_batched_forcing_matches_solo_bitwise():
    """Forced solves of both precisions share one render and one kick sequence per precision."""
    from jathenax_gb300.batch import Batch
    specs = [("turb", 32, "float32", "ppm4", "roe", "rk3", 0.03), ("turb", 70, "float32", "wenoz", "hlle", "rk2", 0.02),
             ("turb", 48, "float64", "ppm4", "roe", "rk3", 0.02), ("turb", 40, "float64", "plm", "llf", "rk4", 0.02),
             ("kh", 40, "float32", "ppm4", "roe", "rk3", 0.02)]
    seeds = [3, 5, 7, 11, 13]
    solves = [make_solve(*spec, tile_y=16, seed=seed) for spec, seed in zip(specs, seeds)]
    Batch(solves).run(steps_per_sync=4)
    for spec, seed, s in zip(specs, seeds, solves):
        alone = make_solve(*spec, tile_y=16, seed=seed)
        alone.run(steps_per_sync=4)
        assert s.state().cycle == alone.state().cycle > 2, spec
        np.testing.assert_array_equal(s.S.cpu().numpy(), alone.S.cpu().numpy(), err_msg=str(spec))


def test_float32_batch_mixing_methods_and_columns_per_lane_is_bitwise():
    """Float32 solves of every reconstruction family in one batch, on marching
    tiles of 1, 2 and 3 columns per lane (short ones on the register path,
    tall ones through the row ring where it is built) and on the
    shared-memory tile: each is bitwise its own solo run (and the solo runs
    agree across tiles)."""
    from jathenax_gb300.batch import Batch, ClockBank
    specs = [("kh", 40, "float32", "dc", "llf", "rk2", 0.03), ("kh", 52, "float32", "wenoz", "hlle", "rk3", 0.02),
             ("smooth", 44, "float32", "ppmx", "roe", "rk4", 0.02), ("turb", 36, "float32", "plm", "hlle", "rk3", 0.03)]
    tiles = [(26, 8), (58, 12), (90, 8), (32, 16), (26, 24), (58, 32), (90, 28)]
    bank = ClockBank(len(specs) * len(tiles))
    solves, expect = [], []
    for i, spec in enumerate(specs):
        for j, (tx, ty) in enumerate(tiles):
            solves.append(make_solve(*spec, tile_y=ty, tile_x=tx, clock=bank.slot(i * len(tiles) + j)))
        expect.append(run_alone(spec, 16, 58))
    Batch(solves, clocks=bank).run(steps_per_sync=4)
    for k, s in enumerate(solves):
        U_alone, t_alone, cyc_alone = expect[k // len(tiles)]
        c = s.state()
        assert (c.time, c.cycle) == (t_alone, cyc_alone), (k, c.time, t_alone)
        np.testing.assert_array_equal(s.S.cpu().numpy(), U_alone, err_msg=f"solve {k}")


def test_lean_four_variable_groups_are_bitwise_solo():
    """Inviscid 4-variable float32 solves on two-column marching tiles form
    lean groups per integrator, which run the packed-pair walk where it is
    used (short tiles, and tall ones with the row ring): each result is
    bitwise its solo run."""
    from jathenax_gb300.batch import Batch, ClockBank
    specs = [("kh", 70, "float32", "ppm4", "roe", "rk3", 0.03), ("kh", 64, "float32", "ppm4", "llf", "rk2", 0.03),
             ("kh", 60, "float32", "plm", "hlle", "rk4", 0.02), ("kh", 66, "float32", "wenoz", "hlle", "rk3", 0.02),
             ("kh", 58, "float32", "ppm4", "roe", "rk4", 0.02), ("kh", 50, "float32", "ppm4", "hlle", "rk3", 0.03)]
    tiles = [(58, 16), (58, 32)]
    bank = ClockBank(len(specs) * len(tiles))
    solves, expect = [], []
    for i, spec in enumerate(specs):
        for j, (tx, ty) in enumerate(tiles):
            solves.append(make_solve(*spec, tile_y=ty, tile_x=tx, clock=bank.slot(i * len(tiles) + j)))
            expect.append(run_alone(spec, ty, tx))
    Batch(solves, clocks=bank).run(steps_per_sync=4)
    for k, (s, (U_alone, t_alone, cyc_alone)) in enumerate(zip(solves, expect)):
        c = s.state()
        assert (c.time, c.cycle) == (t_alone, cyc_alone), (k, c.time, t_alone)
        np.testing.assert_array_equal(s.S.cpu().numpy(), U_alone, err_msg=f"solve {k}")
