"""Host-side logic that needs no GPU: input decks, the OU table, RK schedule."""

from itertools import islice
from pathlib import Path

import numpy as np
import pytest

from jathenax_gb300 import forcing as G
from jathenax_gb300.hydro import RK_STAGES
from jathenax_gb300.input import read_input
from oracle import forcing_oracle as F
from oracle import hydro_oracle as H

DECK = """
[problem]
name = "turbulence"

[mesh]
nx = 256
ny = 256

[time]
integrator = "rk3"
cfl_number = 0.4
tlim = 45.0
nlim = 100000

[hydro]
iso_sound_speed = 1.0
dfloor = 1.17549e-38
reconstruct = "ppm4"
rsolver = "roe"
viscosity = 1.5e-6
smagorinsky_cs = 0.0

[hydro_srcterms]
drag_rate = 0.3333335

[turb_driving]
rseed = 1618
tcorr = 0.75
dt_update = 0.0075
tdriv_start = 0.0
dedt = 0.03703705
nlow = 3
nhigh = 5
npeak = 4
sol_fraction = 1.0
min_kx = -5
max_kx = 5
min_ky = -5
max_ky = 5

[output]
file = "runs/driven_seed1618.npz"
"""


def test_seed1618_deck_equals_defaults(tmp_path):
    path = tmp_path / "turbulence.toml"
    path.write_text(DECK)
    settings = read_input(path)
    defaults = read_input(None, "turbulence")
    defaults["output"]["file"] = "runs/driven_seed1618.npz"
    assert settings == defaults


@pytest.mark.parametrize(("contents", "message"), [
    ("[hydro]\nviscosty = 0", "unknown input setting hydro.viscosty"),
    ("[mesh]\nnx = true", "mesh.nx expects int"),
    ("[turb_driving]\nrseed = 1", "unsupported input section"),
    ("[problem]\nname = \"sod\"", "problem.name must be"),
])
def test_input_rejects_invalid_settings(tmp_path, contents, message):
    path = tmp_path / "input.toml"
    path.write_text(contents)
    with pytest.raises(ValueError, match=message):
        read_input(path)


def test_rk_schedule_matches_oracle():
    assert RK_STAGES == H.RK_TABLE
    # Blend form exactly where the reference uses it (hydro.py:46).
    forms = {k: [H.uses_blend_form(g0, g1) for g0, g1, _, _ in v] for k, v in RK_STAGES.items()}
    assert forms == {"rk2": [False, True], "rk3": [False, True, True],
                     "rk4": [False, False, False, False]}


def test_host_random_streams_match_oracle_bitwise():
    for seed in (0, 1, 1618, 2**31 - 5):
        a = np.fromiter(islice(G.ran_st(seed), 500), float)
        b = np.fromiter(islice(F.uniform_stream(seed), 500), float)
        np.testing.assert_array_equal(a, b)
        a = np.fromiter(islice(G.ran_gaussian_st(seed), 500), float)
        b = np.fromiter(islice(F.gaussian_stream(seed), 500), float)
        np.testing.assert_array_equal(a, b)


def test_host_ou_table_matches_reference_fixture_bitwise(golden):
    g = golden("forcing")
    modes = G.cartesian_modes(3, 5, (-5, 5), (-5, 5))
    np.testing.assert_array_equal(modes, g["modes"])
    table = G.modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, 7)
    np.testing.assert_array_equal(table, g["table"])


@pytest.mark.parametrize("kw", [dict(sol_fraction=0.3), dict(tcorr=0.0), dict(npeak=3.5)])
def test_host_ou_table_variants_match_oracle(kw):
    args = dict(nlow=2, nhigh=4, npeak=3.0, sol_fraction=1.0, rseed=7, tcorr=0.5, dt_update=0.01)
    args.update(kw)
    modes = G.cartesian_modes(args["nlow"], args["nhigh"], (-4, 4), (-4, 4))
    a = G.modal_coefficients(modes, (1.0, 2.0), args["nlow"], args["nhigh"], args["npeak"],
                             args["sol_fraction"], args["rseed"], args["tcorr"], args["dt_update"], 5)
    b = F.ou_table(modes, (1.0, 2.0), args["nlow"], args["nhigh"], args["npeak"],
                   args["sol_fraction"], args["rseed"], args["tcorr"], args["dt_update"], 5)
    np.testing.assert_array_equal(a, b)


def test_forcing_argument_errors():
    with pytest.raises(ValueError, match="1 <= nlow < nhigh"):
        G.cartesian_modes(0, 3, (-3, 3), (-3, 3))
    with pytest.raises(ValueError, match="no Cartesian forcing modes"):
        G.cartesian_modes(8, 9, (-1, 1), (-1, 1))
    modes = G.cartesian_modes(3, 5, (-5, 5), (-5, 5))
    with pytest.raises(ValueError, match="npeak"):
        G.modal_coefficients(modes, (1.0, 1.0), 3, 5, 6.0, 1.0, 1, 0.75, 0.0075, 2)
    with pytest.raises(ValueError, match="tcorr"):
        G.modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1, -1.0, 0.0075, 2)


def test_evolve_argument_errors_before_any_device_work():
    from jathenax_gb300.solver import check_evolve_args
    with pytest.raises(ValueError, match="viscosity must be finite"):
        check_evolve_args(-1.0, 0.0, 0.0, 0.0, None, 1.0, 0.0)
    with pytest.raises(ValueError, match="dedt must be finite"):
        check_evolve_args(0.0, 0.0, 0.0, float("inf"), None, 1.0, 0.0)
    with pytest.raises(ValueError, match="dt_update"):
        check_evolve_args(0.0, 0.0, 0.0, 0.0, object(), 0.0, 0.0)


def test_no_oracle_import_in_package():
    package = Path(__file__).resolve().parents[1] / "jathenax_gb300"
    for path in package.rglob("*.py"):
        text = path.read_text()
        assert "import oracle" not in text and "from oracle" not in text, path


@pytest.mark.parametrize("args", [
    ((1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, 40),
    ((1.0, 2.0), 2, 4, 3.0, 0.3, 7, 0.5, 0.01, 12),
    ((2.0, 1.0), 1, 3, 2.5, 0.0, 2**31 - 5, 0.0, 0.02, 9),
])
def test_native_ou_table_is_bitwise_the_oracle(args):
    lengths, nlow, nhigh = args[0], args[1], args[2]
    modes = G.cartesian_modes(nlow, nhigh, (-nhigh, nhigh), (-nhigh, nhigh))
    native = G.modal_coefficients(modes, *args)
    oracle = F.ou_table(modes, *args)
    np.testing.assert_array_equal(native.view(np.uint64), oracle.view(np.uint64))


def test_precision_guard_estimate():
    """The serving guard's float32 error estimate: measured values for the
    measured sides, side growth above 512, unknown past the measured end
    times, and the promotions it implies."""
    from jathenax_gb300.serve import (FP32_ERR, FP32_ERR_BAR, FP32_ERR_SIDES, FP32_ERR_TLIMS, Request,
                                      fp32_error_estimate, served_dtype)
    assert all(len(rows) == len(FP32_ERR_SIDES) and all(len(r) == len(FP32_ERR_TLIMS) for r in rows)
               for rows in FP32_ERR.values())
    kh_dc, kh_ppm4 = FP32_ERR[("kh", "dc")], FP32_ERR[("kh", "ppm4")]
    # A measured side and end time: that measurement, or a worse one earlier.
    assert fp32_error_estimate("kh", "dc", 128, 0.1) == kh_dc[2][0]
    assert fp32_error_estimate("kh", "dc", 128, 0.2) == max(kh_dc[2][:2])
    # End times between measured ones take the worst up to the next one; sides
    # between measured ones the worse of the two either side.
    assert fp32_error_estimate("kh", "ppm4", 200, 1.2) == max(max(kh_ppm4[2][:5]), max(kh_ppm4[3][:5]))
    assert fp32_error_estimate("kh", "ppm4", 40, 0.3) == max(kh_ppm4[0][:3])
    # Above 512 the estimate grows as side^2 from the 512 row.
    e512 = fp32_error_estimate("kh", "dc", 512, 2.0)
    assert e512 == max(kh_dc[4][:6])
    assert fp32_error_estimate("kh", "dc", 1024, 2.0) == pytest.approx(4 * e512)
    assert fp32_error_estimate("kh", "dc", 100, 3.5) is None
    assert fp32_error_estimate("kh", "unknown", 100, 1.0) is None

    def req(problem, recon, side, tlim, dtype="float32"):
        return Request(rid=0, arrival=0.0, problem=problem, side=side, reconstruct=recon, rsolver="hlle",
                       tlim=tlim, dtype=dtype, seed=1)

    assert served_dtype(req("kh", "ppmx", 64, 0.1)) == "float64"  # PPMX on an under-resolved shear layer
    assert served_dtype(req("kh", "ppmx", 100, 0.1)) == "float64"  # next to side 85
    assert served_dtype(req("kh", "ppmx", 200, 0.2)) == "float32"
    assert served_dtype(req("kh", "ppmx", 200, 0.5)) == "float64"
    assert served_dtype(req("smooth", "dc", 2048, 3.0)) == "float32"
    assert served_dtype(req("kh", "dc", 1976, 2.24)) == "float64"
    assert served_dtype(req("kh", "dc", 1976, 2.24), guard=False) == "float32"
    assert served_dtype(req("kh", "ppmx", 64, 0.1, "float64")) == "float64"
    assert served_dtype(req("smooth", "dc", 64, 0.1), dtype="float64") == "float64"
    assert all(fp32_error_estimate(p, r, s, t) is None or
               (fp32_error_estimate(p, r, s, t) <= FP32_ERR_BAR) == (served_dtype(req(p, r, s, t)) == "float32")
               for (p, r) in FP32_ERR for s in (64, 300, 900) for t in (0.2, 1.1, 2.9))
