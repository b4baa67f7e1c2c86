"""Pin the CPU oracle to the reference: bitwise equality with the golden fixtures.

The fixtures were produced by the unmodified reference package
(tests/golden/make_golden.py); these tests need neither a GPU nor the
reference tree.
"""

from itertools import islice

import numpy as np
import pytest

from oracle import forcing_oracle as F
from oracle import hydro_oracle as H
from oracle import run_oracle as R

RECONS = ("dc", "plm", "ppm4", "ppmx", "wenoz")
SOLVERS = ("llf", "hlle", "roe")
INTEGRATORS = ("rk2", "rk3", "rk4")


@pytest.mark.parametrize("rec", RECONS)
def test_oracle_step_matches_reference_bitwise(golden, rec):
    g = golden("steps")
    U0 = g["U0"]
    for rs in SOLVERS:
        for integ in INTEGRATORS:
            out = H.step(U0, 0.004, 1 / 12, 1 / 10, 1.0, 1e-10, integ, recon=rec, solver=rs)
            np.testing.assert_array_equal(out, g[f"{rec}_{rs}_{integ}"], err_msg=f"{rec}/{rs}/{integ}")


def test_oracle_viscous_smagorinsky_drag_bitwise(golden):
    g = golden("steps")
    for rs in SOLVERS:
        out = H.step(g["U0"], 0.004, 1 / 12, 1 / 10, 1.0, 1e-10, "rk3", nu=2e-3, cs_smag=0.2,
                     drag=0.3, solver=rs)
        np.testing.assert_array_equal(out, g[f"visc_smag_drag_{rs}"])


@pytest.mark.parametrize("pair", [("ppm4", "roe"), ("wenoz", "hlle")])
@pytest.mark.parametrize("integ", INTEGRATORS)
def test_oracle_stage_traces_bitwise(golden, pair, integ):
    g = golden("traces")
    rec, rs = pair
    _, stages = H.step(g["U0"], 0.004, 1 / 12, 1 / 10, 1.0, 1e-10, integ, nu=1e-3, cs_smag=0.1,
                       recon=rec, solver=rs, trace=True)
    for number, stage in enumerate(stages, 1):
        for field, value in stage.items():
            np.testing.assert_array_equal(value, g[f"{rec}_{rs}_{integ}_s{number}_{field}"],
                                          err_msg=f"stage {number} {field}")


def test_oracle_timestep_bitwise(golden):
    g = golden("timestep")
    W = g["W"]
    cases = {"plain": {}, "visc": dict(nu=0.05), "smag": dict(nu=1e-3, cs_smag=2.0),
             "drag": dict(drag=40.0)}
    for name, kw in cases.items():
        assert H.timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, np.inf, 0.0, 1.0, **kw) == g[name]
    assert H.timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, np.inf, 0.999, 1.0) == g["clip"]
    assert H.timestep(W, 1 / 12, 1 / 10, 1.0, 0.4, 1e-4, 0.0, 1.0) == g["growth"]


def test_oracle_forcing_bitwise(golden):
    g = golden("forcing")
    modes = F.forcing_modes(3, 5, (-5, 5), (-5, 5))
    np.testing.assert_array_equal(modes, g["modes"])
    assert len(modes) == 56
    np.testing.assert_array_equal(np.fromiter(islice(F.uniform_stream(1618), 64), float), g["uniforms"])
    np.testing.assert_array_equal(np.fromiter(islice(F.gaussian_stream(1618), 64), float), g["gaussians"])
    table = F.ou_table(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, 7)
    np.testing.assert_array_equal(table, g["table"])
    tables = F.phase_tables(modes, g["x"], g["y"], (1.0, 1.0))
    np.testing.assert_array_equal(F.render(table[2], tables), g["raw"])
    accel = H.normalized_acceleration(g["U"], g["raw"], 0.003, 0.04)
    np.testing.assert_array_equal(accel, g["acceleration"])
    kicked, stages = H.step(g["U"], 0.003, 1 / 16, 1 / 12, 1.0, 1e-10, "rk3", nu=1e-3, drag=0.3,
                            raw_force=g["raw"], dedt=0.04, trace=True)
    np.testing.assert_array_equal(kicked, g["kicked"])
    np.testing.assert_array_equal(stages[-1]["before_kick"], g["before_kick"])


def test_oracle_runs_bitwise(golden):
    g = golden("runs")
    out = R.evolve(g["smooth_U0"], 1 / 64, 1 / 48, 1.0, 1e-10, "rk3", 0.4, 0.2, 100_000)
    np.testing.assert_array_equal(out[0], g["smooth_U"])
    assert out[1] == g["smooth_time"] and out[2] == g["smooth_dt"] and out[3] == g["smooth_cycle"]
    out = R.evolve(g["kh_U0"], 1 / 32, 1 / 32, 1.0, 1e-10, "rk3", 0.4, 0.1, 100_000,
                   recon="wenoz", solver="hlle")
    np.testing.assert_array_equal(out[0], g["kh_U"])
    assert out[3] == g["kh_cycle"]
    x = (np.arange(32) + 0.5) / 32 - 0.5
    tables = F.phase_tables(F.forcing_modes(3, 5, (-5, 5), (-5, 5)), x, x, (1.0, 1.0))
    out = R.evolve(g["turb_U0"], 1 / 32, 1 / 32, 1.0, 1.17549e-38, "rk3", 0.4, 0.5, 12, nu=1.5e-6,
                   drag=0.3333335, forcing=(g["turb_table"], tables), dt_update=0.0075, dedt=0.03703705)
    np.testing.assert_array_equal(out[0], g["turb_U"])
    assert out[1] == g["turb_time"] and out[3] == g["turb_cycle"]


def test_oracle_sgs_hook_bitwise(golden):
    g = golden("sgs")
    final, stages = H.step(g["U"], 0.01, 1 / 8, 1 / 8, 1.0, 1e-10, "rk3", trace=True,
                           stress=lambda w, W: w * W, stress_args=g["scale"])
    np.testing.assert_array_equal(final, g["final"])
    for number, stage in enumerate(stages, 1):
        np.testing.assert_array_equal(stage["flux_x"], g[f"s{number}_flux_x"])


def test_oracle_rejects_bad_predictor():
    U = np.ones((6, 8, 3))
    with pytest.raises(ValueError, match="predict_stress must return"):
        H.step(U, 0.01, 1 / 8, 1 / 6, 1.0, 1e-10, "rk3", stress=lambda w, W: W[:1])


def test_reference_suite_passed_when_fixtures_were_made(golden):
    summary = str(golden("steps")["meta_reference_tests"])
    assert "passed" in summary and "failed" not in summary, summary
