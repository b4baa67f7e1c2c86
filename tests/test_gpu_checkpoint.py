"""Checkpoint/resume: a run written to npz and resumed in a new Solve continues
bitwise as the uninterrupted run (state, time, cycle), whether it stopped at
its cycle limit or was cut between graph replays with a step still pending."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(kind, dtype, nlim, tlim=1.0):
    import torch
    from jathenax_gb300.forcing import cartesian_modes, forcing_basis, modal_coefficients
    from jathenax_gb300.initial_conditions import cell_centers, kelvin_helmholtz_tanh, uniform_rest
    from jathenax_gb300.solver import Solve
    td = getattr(torch, dtype)
    if kind == "kh":
        return Solve(kelvin_helmholtz_tanh(48, 40), 1 / 48, 1 / 40, 1.0, 1e-10, "rk3", 0.4, tlim, nlim, dtype=td)
    if kind == "smagorinsky_rk4":
        return Solve(kelvin_helmholtz_tanh(40, 40)[..., :3], 1 / 40, 1 / 40, 1.0, 1e-10, "rk4", 0.4, tlim, nlim,
                     viscosity=1e-4, smagorinsky_cs=0.17, drag_rate=0.2, reconstruct="wenoz", rsolver="hlle",
                     dtype=td)
    n = 36
    x, _ = cell_centers(n, n)
    modes = cartesian_modes(3, 5, (-5, 5), (-5, 5))
    table = modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, int(np.ceil(tlim / 0.0075)) + 1)
    return Solve(uniform_rest(n, n), 1 / n, 1 / n, 1.0, 1.17549e-38, "rk3", 0.4, tlim, nlim, viscosity=1.5e-6,
                 drag_rate=0.3333335, forcing=(table, forcing_basis(modes, x, x, (1.0, 1.0))), dt_update=0.0075,
                 dedt=0.03703705, dtype=td)


def finish(solve):
    solve.run(steps_per_sync=4)
    c = solve.state()
    return solve.S.cpu().numpy(), c.time, c.cycle


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("kind", ["kh", "turbulence", "smagorinsky_rk4"])
def test_resume_after_the_cycle_limit_is_bitwise(tmp_path, kind, dtype):
    U_full, t_full, c_full = finish(make(kind, dtype, 30))
    first = make(kind, dtype, 13)
    first.run(steps_per_sync=4, checkpoint=tmp_path / "c.npz")
    saved = np.load(tmp_path / "c.npz")
    assert int(saved["cycle"]) == 13 and saved["conserved"].dtype == np.dtype(dtype)
    second = make(kind, dtype, 30)
    second.resume(tmp_path / "c.npz")
    U, t, c = finish(second)
    assert c == c_full == 30 and t == t_full, kind
    np.testing.assert_array_equal(U, U_full)


@pytest.mark.parametrize("kind", ["kh", "turbulence"])
def test_resume_between_steps_with_a_pending_cycle_is_bitwise(tmp_path, kind):
    U_full, t_full, c_full = finish(make(kind, "float64", 25))
    first = make(kind, "float64", 25)
    for _ in range(11):
        first.enqueue_step()
    first.checkpoint(tmp_path / "mid.npz")
    second = make(kind, "float64", 25)
    second.resume(tmp_path / "mid.npz")
    U, t, c = finish(second)
    assert c == c_full == 25 and t == t_full
    np.testing.assert_array_equal(U, U_full)


def test_resume_rejects_a_different_problem(tmp_path):
    first = make("kh", "float64", 3)
    first.run(steps_per_sync=4, checkpoint=tmp_path / "c.npz")
    with pytest.raises(ValueError, match="different problem description"):
        make("smagorinsky_rk4", "float64", 5).resume(tmp_path / "c.npz")
    with pytest.raises(ValueError, match="different problem description"):
        make("kh", "float32", 5).resume(tmp_path / "c.npz")


def test_evolve_isothermal_checkpoints_and_resumes(tmp_path):
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    from jathenax_gb300.run import evolve_isothermal
    U0 = kelvin_helmholtz_tanh(32, 32)
    args = (1 / 32, 1 / 32, 1.0, 1e-10, "rk3", 0.4, 1.0)
    U_full, t_full, _, c_full = evolve_isothermal(U0, *args, 20)
    evolve_isothermal(U0, *args, 9, checkpoint=tmp_path / "run.npz")
    U, t, _, c = evolve_isothermal(U0, *args, 20, resume=tmp_path / "run.npz")
    assert c == c_full == 20 and t == t_full
    np.testing.assert_array_equal(U, U_full)


def test_overlapped_host_advance_equals_one_at_a_time():
    """advance_host_many overlaps transfers with cycles; results must equal advance_host in turn."""
    import torch
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh
    from jathenax_gb300.solver import Solve
    rng = np.random.default_rng(4)
    base = kelvin_helmholtz_tanh(96, 80)
    states = [torch.from_numpy(base * (1 + 0.01 * rng.standard_normal(base.shape))).pin_memory() for _ in range(5)]
    a = Solve(base, 1 / 96, 1 / 80, 1.0, 1e-10, "rk3", 0.4, 10.0, 10**6)
    b = Solve(base, 1 / 96, 1 / 80, 1.0, 1e-10, "rk3", 0.4, 10.0, 10**6)
    outs_a = [torch.empty_like(x).pin_memory() for x in states]
    outs_b = [torch.empty_like(x).pin_memory() for x in states]
    for x, o in zip(states, outs_a):
        a.advance_host(x, o, steps=2)
    b.advance_host_many(states, outs_b, steps=2)
    torch.cuda.synchronize()
    for x, y in zip(outs_a, outs_b):
        np.testing.assert_array_equal(x.numpy(), y.numpy())
    assert a.state().cycle == b.state().cycle and a.state().time == b.state().time
