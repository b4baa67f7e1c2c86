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


def main(argv=None):
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("problem", nargs="?", choices=PROBLEMS)
    parser.add_argument("-i", "--input", type=Path, help="TOML input deck")
    parser.add_argument("--nx", type=int, help="Number of x cells")
    parser.add_argument("--ny", type=int, help="Number of y cells")
    parser.add_argument("--tlim", type=float, help="Stop time")
    parser.add_argument("--integrator", choices=("rk2", "rk3", "rk4"))
    parser.add_argument("--reconstruct", choices=RECONSTRUCTIONS, help="Face reconstruction (default: ppm4)")
    parser.add_argument("--rsolver", choices=RIEMANN_SOLVERS, help="Riemann solver (default: roe)")
    parser.add_argument("--viscosity", type=float, help="Uniform kinematic viscosity")
    parser.add_argument("--smagorinsky-cs", type=float)
    parser.add_argument("--sgs-model", help="Python module with load_weights and predict_stress")
    parser.add_argument("--sgs-weights", type=Path, help="Checkpoint passed to load_weights")
    parser.add_argument("--output", type=Path, help="Output .npz file")
    parser.add_argument("--precision", choices=("float64", "float32"), default="float64",
                        help="State precision on the GPU (default: float64)")
    parser.add_argument("--checkpoint", type=Path,
                        help="Write a resumable checkpoint npz here (every --checkpoint-every cycles and at the end)")
    parser.add_argument("--checkpoint-every", type=int, default=0, help="Cycles between checkpoints")
    parser.add_argument("--resume", type=Path, help="Continue from a checkpoint of the same problem")
    args = parser.parse_args(argv)
    try:
        settings = read_input(args.input, args.problem)
    except (OSError, ValueError) as error:
        parser.error(str(error))

    mesh, time_cfg, hydro = settings["mesh"], settings["time"], settings["hydro"]
    for section, keys in ((mesh, ("nx", "ny")), (time_cfg, ("tlim", "integrator")),
                          (hydro, ("reconstruct", "rsolver", "viscosity", "smagorinsky_cs"))):
        for key in keys:
            value = getattr(args, key)
            if value is not None:
                section[key] = value
    problem = settings["problem"]["name"]
    model_name = args.sgs_model if args.sgs_model is not None else settings["sgs"]["model"]
    checkpoint = args.sgs_weights
    if checkpoint is None and settings["sgs"]["weights"]:
        checkpoint = Path(settings["sgs"]["weights"])
    if checkpoint is not None and not model_name:
        parser.error("SGS weights require a model (sgs.model or --sgs-model)")

    nx, ny = mesh["nx"], mesh["ny"]
    tlim, nlim, cfl = time_cfg["tlim"], time_cfg["nlim"], time_cfg["cfl_number"]
    integrator = time_cfg["integrator"]
    reconstruct, rsolver = hydro["reconstruct"], hydro["rsolver"]
    cs, dfloor = hydro["iso_sound_speed"], hydro["dfloor"]
    viscosity, smagorinsky_cs = hydro["viscosity"], hydro["smagorinsky_cs"]
    drag_rate = settings["hydro_srcterms"]["drag_rate"]
    if min(nx, ny) < 6:
        parser.error("each grid dimension must be at least six")
    if not 1 <= nlim <= np.iinfo(np.int32).max:
        parser.error("time.nlim must be a positive 32-bit cycle limit")
    for key, value in (("time.tlim", tlim), ("time.cfl_number", cfl),
                       ("hydro.iso_sound_speed", cs), ("hydro.dfloor", dfloor)):
        if not isfinite(value) or value <= 0:
            parser.error(f"{key} must be finite and positive")
    if integrator not in ("rk2", "rk3", "rk4"):
        parser.error("time.integrator must be rk2, rk3, or rk4")
    if reconstruct not in RECONSTRUCTIONS or rsolver not in RIEMANN_SOLVERS:
        parser.error("invalid hydro.reconstruct or hydro.rsolver")
    output = args.output or Path(settings["output"]["file"])
    if output.suffix != ".npz":
        parser.error("--output must end in .npz")

    dx, dy = 1.0 / nx, 1.0 / ny
    x, y = cell_centers(nx, ny)
    forcing = None
    dt_update, tdriv_start, dedt = 1.0, 0.0, 0.0
    if problem == "turbulence":
        driving = settings["turb_driving"]
        dt_update, tdriv_start, dedt = (driving[k] for k in ("dt_update", "tdriv_start", "dedt"))
        if not (0 < dt_update < np.inf and isfinite(tdriv_start)):
            parser.error("forcing requires finite tdriv_start and positive finite dt_update")
        U_initial = uniform_rest(nx, ny)
        modes = cartesian_modes(driving["nlow"], driving["nhigh"],
                                (driving["min_kx"], driving["max_kx"]),
                                (driving["min_ky"], driving["max_ky"]))
        updates = int(np.ceil(max(0.0, tlim - tdriv_start) / dt_update)) + 1
        coefficients = modal_coefficients(
            modes, (1.0, 1.0), driving["nlow"], driving["nhigh"], driving["npeak"],
            driving["sol_fraction"], driving["rseed"], driving["tcorr"], dt_update, updates)
        forcing = (coefficients, forcing_basis(modes, x, y, (1.0, 1.0)))
    elif problem == "kh":
        U_initial = kelvin_helmholtz(x, y)
    else:
        U_initial = smooth_waves(nx, ny)
    state_dtype = np.float32 if args.precision == "float32" else np.float64
    U_initial = U_initial.astype(state_dtype)

    predict_stress, sgs_weights = None, None
    if model_name:
        model = import_module(model_name)
        predict_stress = model.predict_stress
        sgs_weights = model.load_weights(checkpoint)

    U, time, dt, cycle = evolve_isothermal(
        U_initial, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim,
        viscosity=viscosity, smagorinsky_cs=smagorinsky_cs, drag_rate=drag_rate,
        forcing=forcing, dt_update=dt_update, tdriv_start=tdriv_start, dedt=dedt,
        reconstruct=reconstruct, rsolver=rsolver,
        predict_stress=predict_stress, sgs_weights=sgs_weights,
        checkpoint=args.checkpoint, checkpoint_every=args.checkpoint_every, resume=args.resume)
    reached_tlim = time == np.float64(tlim)
    if not np.isfinite(U).all() or not np.isfinite(time) or (not reached_tlim and cycle != nlim):
        raise RuntimeError(f"Periodic run ended at t={time} after {cycle} steps")

    output.parent.mkdir(parents=True, exist_ok=True)
    np.savez(output, x=x, y=y, initial=U_initial, conserved=U, time=time, dt=dt, cycle=cycle,
             problem=problem, sgs_model=model_name)
    drift = (U.sum(axis=(0, 1), dtype=np.float64)
             - U_initial.sum(axis=(0, 1), dtype=np.float64)) * dx * dy
    name = _lib.torch().cuda.get_device_name()
    print(f"{integrator.upper()} on {name}, {U.dtype}, {cycle} steps to t={time:.6g}")
    if not reached_tlim:
        print(f"Reached time.nlim={nlim} before tlim={tlim:g}")
    print(f"Reconstruction {reconstruct}, Riemann solver {rsolver}")
    print(f"Change in box mass and momenta {drift[:3]}")
    if U.shape[-1] > 3:
        print(f"Change in integrated tracer {drift[3:]}")
    print(output.resolve())


if __name__ == "__main__":
    main()
