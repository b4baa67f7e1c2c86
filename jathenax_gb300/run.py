"""Run a periodic isothermal problem on the GPU (drop-in for jathenax/run.py).

``evolve_isothermal`` keeps the reference signature (run.py:24-27) and
returns ``(U, time, dt, cycle)``. The command line takes the same problem
names, ``-i deck.toml`` and flags, and writes the same npz keys.
"""

import argparse
from importlib import import_module
from math import isfinite
from pathlib import Path

import numpy as np

from . import _lib
from .fluxes import RECONSTRUCTIONS, RIEMANN_SOLVERS
from .forcing import cartesian_modes, forcing_basis, modal_coefficients
from .initial_conditions import cell_centers, kelvin_helmholtz, smooth_waves, uniform_rest
from .input import PROBLEMS, read_input
from .solver import Solve, check_evolve_args


def evolve_isothermal(U, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim, *,
                      viscosity=0.0, smagorinsky_cs=0.0, drag_rate=0.0,
                      forcing=None, dt_update=1.0, tdriv_start=0.0, dedt=0.0,
                      reconstruct="ppm4", rsolver="roe", predict_stress=None, sgs_weights=None,
                      steps_per_sync=32, checkpoint=None, checkpoint_every=0, resume=None):
    """Advance the device-resident periodic grid to tlim or nlim cycles (run.py:20-69).

    ``forcing`` is ``(coefficients, basis)`` from modal_coefficients and
    forcing_basis. Time and dt are accumulated in float64 on the device.
    Added (no reference counterpart): ``resume`` continues from a checkpoint
    npz of the same problem instead of from U; ``checkpoint`` writes one
    every ``checkpoint_every`` cycles and at the end (Solve.checkpoint).
    """
    check_evolve_args(viscosity, smagorinsky_cs, drag_rate, dedt, forcing, dt_update, tdriv_start)
    solve = Solve(U, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim, viscosity=viscosity,
                  smagorinsky_cs=smagorinsky_cs, drag_rate=drag_rate, forcing=forcing,
                  dt_update=dt_update, tdriv_start=tdriv_start, dedt=dedt,
                  reconstruct=reconstruct, rsolver=rsolver, predict_stress=predict_stress,
                  sgs_weights=sgs_weights)
    if resume is not None:
        solve.resume(resume)
    solve.run(steps_per_sync=steps_per_sync, checkpoint=checkpoint, checkpoint_every=checkpoint_every)
    S, time, dt, cycle = solve.result()
    if _lib.is_device_array(U):
        t = _lib.torch()
        f64 = dict(dtype=t.float64, device=S.device)
        return S, t.tensor(time, **f64), t.tensor(dt, **f64), t.tensor(cycle, dtype=t.int32, device=S.device)
    return S.cpu().numpy(), np.float64(time), np.float64(dt), np.int32(cycle)


# ---------------------------------------------------------------------------
# Command line (run.py:72-195): the reference's flags, deck precedence, error
# messages, npz keys and printed summary, organised as tables: the flags, the
# deck section each command-line override lands in, the checks (in the order
# the reference applies them, so the first error reported is the same), and
# one set-up function per problem.
# ---------------------------------------------------------------------------
_INTEGRATORS = ("rk2", "rk3", "rk4")
_FLAGS = (
    (("problem",), dict(nargs="?", choices=PROBLEMS)),
    (("-i", "--input"), dict(type=Path, help="TOML input deck")),
    (("--nx",), dict(type=int, help="Number of x cells")),
    (("--ny",), dict(type=int, help="Number of y cells")),
    (("--tlim",), dict(type=float, help="Stop time")),
    (("--integrator",), dict(choices=_INTEGRATORS)),
    (("--reconstruct",), dict(choices=RECONSTRUCTIONS, help="Face reconstruction (default: ppm4)")),
    (("--rsolver",), dict(choices=RIEMANN_SOLVERS, help="Riemann solver (default: roe)")),
    (("--viscosity",), dict(type=float, help="Uniform kinematic viscosity")),
    (("--smagorinsky-cs",), dict(type=float)),
    (("--sgs-model",), dict(help="Python module with load_weights and predict_stress")),
    (("--sgs-weights",), dict(type=Path, help="Checkpoint passed to load_weights")),
    (("--output",), dict(type=Path, help="Output .npz file")),
    # Added here (no reference counterpart):
    (("--precision",), dict(choices=("float64", "float32"), default="float64",
                            help="State precision on the GPU (default: float64)")),
    (("--checkpoint",), dict(type=Path, help="Write a resumable checkpoint npz here "
                                             "(every --checkpoint-every cycles and at the end)")),
    (("--checkpoint-every",), dict(type=int, default=0, help="Cycles between checkpoints")),
    (("--resume",), dict(type=Path, help="Continue from a checkpoint of the same problem")),
)
# command-line override -> deck section it replaces
_OVERRIDES = {"nx": "mesh", "ny": "mesh", "tlim": "time", "integrator": "time", "reconstruct": "hydro",
              "rsolver": "hydro", "viscosity": "hydro", "smagorinsky_cs": "hydro"}


def _finite_positive(value):
    return isfinite(value) and value > 0


# (test of the merged settings, message when it fails), in the reference's order.
_CHECKS = (
    (lambda s: min(s["mesh"]["nx"], s["mesh"]["ny"]) >= 6, "each grid dimension must be at least six"),
    (lambda s: 1 <= s["time"]["nlim"] <= np.iinfo(np.int32).max,
     "time.nlim must be a positive 32-bit cycle limit"),
    (lambda s: _finite_positive(s["time"]["tlim"]), "time.tlim must be finite and positive"),
    (lambda s: _finite_positive(s["time"]["cfl_number"]), "time.cfl_number must be finite and positive"),
    (lambda s: _finite_positive(s["hydro"]["iso_sound_speed"]), "hydro.iso_sound_speed must be finite and positive"),
    (lambda s: _finite_positive(s["hydro"]["dfloor"]), "hydro.dfloor must be finite and positive"),
    (lambda s: s["time"]["integrator"] in _INTEGRATORS, "time.integrator must be rk2, rk3, or rk4"),
    (lambda s: s["hydro"]["reconstruct"] in RECONSTRUCTIONS and s["hydro"]["rsolver"] in RIEMANN_SOLVERS,
     "invalid hydro.reconstruct or hydro.rsolver"),
)


def _driven_setup(settings, x, y):
    """Rest state plus the OU forcing tables of [turb_driving] (run.py:138-155)."""
    drive = settings["turb_driving"]
    dt_update, t_start = drive["dt_update"], drive["tdriv_start"]
    if not (0 < dt_update < np.inf and isfinite(t_start)):
        raise ValueError("forcing requires finite tdriv_start and positive finite dt_update")
    band = (drive["nlow"], drive["nhigh"])
    modes = cartesian_modes(*band, (drive["min_kx"], drive["max_kx"]), (drive["min_ky"], drive["max_ky"]))
    updates = int(np.ceil(max(0.0, settings["time"]["tlim"] - t_start) / dt_update)) + 1
    table = modal_coefficients(modes, (1.0, 1.0), *band, drive["npeak"], drive["sol_fraction"],
                               drive["rseed"], drive["tcorr"], dt_update, updates)
    forcing = dict(forcing=(table, forcing_basis(modes, x, y, (1.0, 1.0))), dt_update=dt_update,
                   tdriv_start=t_start, dedt=drive["dedt"])
    return uniform_rest(len(x), len(y)), forcing


# problem -> set-up returning (initial conserved state, forcing keywords)
_PROBLEM_SETUP = {
    "turbulence": _driven_setup,
    "kh": lambda settings, x, y: (kelvin_helmholtz(x, y), {}),
    "smooth": lambda settings, x, y: (smooth_waves(len(x), len(y)), {}),
}


def _merged_settings(args, fail):
    """Problem defaults < deck < command line, then the reference's checks."""
    try:
        settings = read_input(args.input, args.problem)
    except (OSError, ValueError) as error:
        fail(str(error))
    for key, section in _OVERRIDES.items():
        value = getattr(args, key)
        if value is not None:
            settings[section][key] = value
    return settings


def _sgs_choice(args, settings, fail):
    """(module name, weights path or None); weights need a model (run.py:103-108)."""
    model = args.sgs_model if args.sgs_model is not None else settings["sgs"]["model"]
    weights = args.sgs_weights
    if weights is None and settings["sgs"]["weights"]:
        weights = Path(settings["sgs"]["weights"])
    if weights is not None and not model:
        fail("SGS weights require a model (sgs.model or --sgs-model)")
    return model, weights


def _report(setup, U, U_initial, time, cycle, output):
    """The reference's summary lines (run.py:186-195), float64 box drift."""
    drift = (U.sum(axis=(0, 1), dtype=np.float64)
             - U_initial.sum(axis=(0, 1), dtype=np.float64)) * setup["dx"] * setup["dy"]
    device = _lib.torch().cuda.get_device_name()
    lines = [f"{setup['integrator'].upper()} on {device}, {U.dtype}, {cycle} steps to t={time:.6g}"]
    if not setup["reached_tlim"]:
        lines.append(f"Reached time.nlim={setup['nlim']} before tlim={setup['tlim']:g}")
    lines.append(f"Reconstruction {setup['reconstruct']}, Riemann solver {setup['rsolver']}")
    lines.append(f"Change in box mass and momenta {drift[:3]}")
    if U.shape[-1] > 3:
        lines.append(f"Change in integrated tracer {drift[3:]}")
    lines.append(str(output.resolve()))
    print("\n".join(lines))


def main(argv=None):
    parser = argparse.ArgumentParser(description=__doc__)
    for names, options in _FLAGS:
        parser.add_argument(*names, **options)
    args = parser.parse_args(argv)
    settings = _merged_settings(args, parser.error)
    model_name, weights_path = _sgs_choice(args, settings, parser.error)
    for test, message in _CHECKS:
        if not test(settings):
            parser.error(message)
    output = args.output or Path(settings["output"]["file"])
    if output.suffix != ".npz":
        parser.error("--output must end in .npz")

    mesh, clock, gas = settings["mesh"], settings["time"], settings["hydro"]
    problem = settings["problem"]["name"]
    nx, ny = mesh["nx"], mesh["ny"]
    x, y = cell_centers(nx, ny)
    try:
        U_initial, forcing = _PROBLEM_SETUP[problem](settings, x, y)
    except ValueError as error:
        parser.error(str(error))
    U_initial = U_initial.astype(np.float32 if args.precision == "float32" else np.float64)

    hook = {}
    if model_name:
        model = import_module(model_name)
        hook = dict(predict_stress=model.predict_stress, sgs_weights=model.load_weights(weights_path))

    U, time, dt, cycle = evolve_isothermal(
        U_initial, 1.0 / nx, 1.0 / ny, gas["iso_sound_speed"], gas["dfloor"], clock["integrator"],
        clock["cfl_number"], clock["tlim"], clock["nlim"], viscosity=gas["viscosity"],
        smagorinsky_cs=gas["smagorinsky_cs"], drag_rate=settings["hydro_srcterms"]["drag_rate"],
        reconstruct=gas["reconstruct"], rsolver=gas["rsolver"], checkpoint=args.checkpoint,
        checkpoint_every=args.checkpoint_every, resume=args.resume, **forcing, **hook)
    reached_tlim = time == np.float64(clock["tlim"])
    if not np.isfinite(U).all() or not np.isfinite(time) or (not reached_tlim and cycle != clock["nlim"]):
        raise RuntimeError(f"Periodic run ended at t={time} after {cycle} steps")

    output.parent.mkdir(parents=True, exist_ok=True)
    np.savez(output, x=x, y=y, initial=U_initial, conserved=U, time=time, dt=dt, cycle=cycle,
             problem=problem, sgs_model=model_name)
    _report(dict(dx=1.0 / nx, dy=1.0 / ny, integrator=clock["integrator"], nlim=clock["nlim"],
                 tlim=clock["tlim"], reached_tlim=reached_tlim, reconstruct=gas["reconstruct"],
                 rsolver=gas["rsolver"]), U, U_initial, time, cycle, output)


if __name__ == "__main__":
    main()
