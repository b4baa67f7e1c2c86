"""Generate the golden fixtures in this directory from the JathenAX reference itself.

Usage (needs the reference source tree, e.g. a checkout of JathenAX):

    python tests/golden/make_golden.py --reference <path-to-JathenAX-checkout>

JathenAX needs jax/jaxlib, which are not installable here, so the reference's
unmodified package is imported on top of ``oracle/jaxshim`` (a NumPy-backed
stand-in for the jax API it uses, float64 throughout). Before writing any
fixture this script runs the reference's own test suite under the shim and
stops if it does not pass, so the fixtures come from a validated runner.

The fixtures are small (.npz, < 1 MB in total) and are what the CPU oracle and
the GPU kernels are checked against in ``tests/``; nothing at test time reads
the reference tree.
"""

import argparse
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
SHIM = REPO / "oracle" / "jaxshim"


def run_reference_tests(reference):
    env = dict(os.environ, PYTHONPATH=f"{SHIM}{os.pathsep}{reference}", PYTHONDONTWRITEBYTECODE="1")
    result = subprocess.run(
        [sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", str(reference / "tests")],
        cwd="/tmp", env=env, capture_output=True, text=True)
    tail = result.stdout.strip().splitlines()[-1] if result.stdout.strip() else ""
    if result.returncode != 0:
        sys.exit(f"reference tests failed under the shim:\n{result.stdout}\n{result.stderr}")
    return tail


def noisy_kh(nx, ny, seed, extra_scalar=False):
    from jathenax.initial_conditions import kelvin_helmholtz
    x = (np.arange(nx) + 0.5) / nx - 0.5
    y = (np.arange(ny) + 0.5) / ny - 0.5
    U = kelvin_helmholtz(x, y)
    rng = np.random.default_rng(seed)
    U = U + 0.05 * rng.standard_normal(U.shape)
    U[..., 0] = 1.0 + 0.2 * np.abs(rng.standard_normal(U.shape[:2]))
    if extra_scalar:
        U = np.concatenate((U, 0.3 * U[..., :1] * rng.random(U.shape[:2] + (1,))), axis=-1)
    return U


def main():
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--reference", type=Path, required=True)
    args = parser.parse_args()
    reference = args.reference.resolve()
    summary = run_reference_tests(reference)
    print("reference tests under the shim:", summary)

    sys.path[:0] = [str(SHIM), str(reference)]
    import jax.numpy as jnp
    from jathenax import forcing, hydro, run
    from jathenax.fluxes import RECONSTRUCTIONS, RIEMANN_SOLVERS

    meta = dict(reference_tests=summary, generator="tests/golden/make_golden.py")

    # 1. One step for every reconstruction x solver x integrator (12 x 10, 4 vars).
    U0 = noisy_kh(12, 10, seed=1)
    dx, dy, dt = 1 / 12, 1 / 10, 0.004
    steps = {"U0": U0}
    for rec in RECONSTRUCTIONS:
        for rs in RIEMANN_SOLVERS:
            for integ in hydro.RK_STAGES:
                out = hydro.isothermal_step(jnp.asarray(U0), dt, dx, dy, 1.0, 1e-10, integ,
                                            reconstruct=rec, rsolver=rs)
                steps[f"{rec}_{rs}_{integ}"] = np.asarray(out)
    # Viscous, Smagorinsky and drag with all solvers (RK3, ppm4).
    for rs in RIEMANN_SOLVERS:
        out = hydro.isothermal_step(jnp.asarray(U0), dt, dx, dy, 1.0, 1e-10, "rk3",
                                    viscosity=2e-3, smagorinsky_cs=0.2, drag_rate=0.3, rsolver=rs)
        steps[f"visc_smag_drag_{rs}"] = np.asarray(out)
    np.savez_compressed(HERE / "steps.npz", **steps, **{f"meta_{k}": v for k, v in meta.items()})

    # 2. Full per-stage traces for ppm4/roe and wenoz/hlle with every integrator.
    traces = {"U0": U0}
    for rec, rs in (("ppm4", "roe"), ("wenoz", "hlle")):
        for integ in hydro.RK_STAGES:
            _, stages = hydro.isothermal_step(jnp.asarray(U0), dt, dx, dy, 1.0, 1e-10, integ,
                                              viscosity=1e-3, smagorinsky_cs=0.1,
                                              reconstruct=rec, rsolver=rs, trace=True)
            for number, stage in enumerate(stages, 1):
                for field, value in stage.items():
                    traces[f"{rec}_{rs}_{integ}_s{number}_{field}"] = np.asarray(value)
    np.savez_compressed(HERE / "traces.npz", **traces)

    # 3. Timestep limits.
    from jathenax.hydro import isothermal_timestep, recover_isothermal
    _, W = recover_isothermal(jnp.asarray(U0), 1e-10)
    dts = {"W": np.asarray(W)}
    cases = {"plain": {}, "visc": dict(viscosity=0.05), "smag": dict(viscosity=1e-3, smagorinsky_cs=2.0),
             "drag": dict(drag_rate=40.0)}
    for name, kw in cases.items():
        dts[name] = np.asarray(isothermal_timestep(W, dx, dy, 1.0, 0.4, np.inf, 0.0, 1.0, **kw))
    dts["clip"] = np.asarray(isothermal_timestep(W, dx, dy, 1.0, 0.4, np.inf, 0.999, 1.0))
    dts["growth"] = np.asarray(isothermal_timestep(W, dx, dy, 1.0, 0.4, 1e-4, 0.0, 1.0))
    np.savez_compressed(HERE / "timestep.npz", **dts)

    # 4. Forcing, seed-1618 deck: draws, modes, OU table rows, render, normalise.
    modes = forcing.cartesian_modes(3, 5, (-5, 5), (-5, 5))
    from itertools import islice
    uniforms = np.fromiter(islice(forcing.ran_st(1618), 64), float)
    gaussians = np.fromiter(islice(forcing.ran_gaussian_st(1618), 64), float)
    table = forcing.modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, 7)
    nx, ny = 16, 12
    x = (np.arange(nx) + 0.5) / nx - 0.5
    y = (np.arange(ny) + 0.5) / ny - 0.5
    basis = forcing.forcing_basis(jnp.asarray(modes), jnp.asarray(x), jnp.asarray(y), (1.0, 1.0))
    raw = np.asarray(forcing.render_force(jnp.asarray(table[2]), basis))
    Uf = noisy_kh(nx, ny, seed=2)[..., :3]
    accel = np.asarray(forcing.normalize_force(jnp.asarray(Uf), jnp.asarray(raw), 0.003, 0.04))
    kicked, kstages = hydro.isothermal_step(jnp.asarray(Uf), 0.003, 1 / nx, 1 / ny, 1.0, 1e-10, "rk3",
                                            viscosity=1e-3, drag_rate=0.3, raw_force=jnp.asarray(raw),
                                            dedt=0.04, trace=True)
    np.savez_compressed(
        HERE / "forcing.npz", modes=modes, uniforms=uniforms, gaussians=gaussians, table=table,
        x=x, y=y, raw=raw, U=Uf, acceleration=accel, kicked=np.asarray(kicked),
        before_kick=np.asarray(kstages[-1]["before_kick"]),
        kick_acceleration=np.asarray(kstages[-1]["acceleration"]))

    # 5. Whole runs: the smooth problem (64x48, ppm4/roe/rk3, cfl 0.4, t=0.2),
    #    a short Kelvin-Helmholtz run and a short forced turbulence run.
    from jathenax.initial_conditions import kelvin_helmholtz
    runs = {}
    nx, ny = 64, 48
    x = (np.arange(nx) + 0.5) / nx - 0.5
    y = (np.arange(ny) + 0.5) / ny - 0.5
    px, py = np.meshgrid(2.0 * np.pi * x, 2.0 * np.pi * y)
    rho = 1.0 + 0.1 * np.sin(px + py)
    U = np.stack((rho, rho * 0.2 * np.cos(py), rho * 0.2 * np.sin(px)), axis=-1)
    out = run.evolve_isothermal(jnp.asarray(U), 1 / nx, 1 / ny, 1.0, 1e-10, "rk3", 0.4, 0.2, 100_000)
    runs.update(smooth_U0=U, smooth_U=np.asarray(out[0]), smooth_time=np.asarray(out[1]),
                smooth_dt=np.asarray(out[2]), smooth_cycle=np.asarray(out[3]))
    nx = ny = 32
    x = (np.arange(nx) + 0.5) / nx - 0.5
    U = kelvin_helmholtz(x, x)
    out = run.evolve_isothermal(jnp.asarray(U), 1 / nx, 1 / ny, 1.0, 1e-10, "rk3", 0.4, 0.1, 100_000,
                                reconstruct="wenoz", rsolver="hlle")
    runs.update(kh_U0=U, kh_U=np.asarray(out[0]), kh_time=np.asarray(out[1]),
                kh_dt=np.asarray(out[2]), kh_cycle=np.asarray(out[3]))
    U = np.zeros((ny, nx, 3))
    U[..., 0] = 1.0
    updates = int(np.ceil(0.5 / 0.0075)) + 1
    table = forcing.modal_coefficients(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, updates)
    basis = forcing.forcing_basis(jnp.asarray(modes), jnp.asarray(x), jnp.asarray(x), (1.0, 1.0))
    out = run.evolve_isothermal(jnp.asarray(U), 1 / nx, 1 / ny, 1.0, 1.17549e-38, "rk3", 0.4, 0.5, 12,
                                viscosity=1.5e-6, drag_rate=0.3333335,
                                forcing=(jnp.asarray(table), basis), dt_update=0.0075,
                                tdriv_start=0.0, dedt=0.03703705)
    runs.update(turb_U0=U, turb_table=table, turb_U=np.asarray(out[0]), turb_time=np.asarray(out[1]),
                turb_dt=np.asarray(out[2]), turb_cycle=np.asarray(out[3]))
    np.savez_compressed(HERE / "runs.npz", **runs)

    # 6. The SGS hook: a stress proportional to the primitives, traced.
    U = noisy_kh(8, 8, seed=3)
    scale = np.asarray([0.0125, 0.025, -0.0375])
    final, stages = hydro.isothermal_step(
        jnp.asarray(U), 0.01, 1 / 8, 1 / 8, 1.0, 1e-10, "rk3", trace=True,
        predict_stress=lambda w, W: w * W, sgs_weights=jnp.asarray(scale))
    np.savez_compressed(HERE / "sgs.npz", U=U, scale=scale, final=np.asarray(final),
                        **{f"s{n}_{k}": np.asarray(v) for n, s in enumerate(stages, 1)
                           for k, v in s.items() if k in ("flux_x", "flux_y", "primitives")})
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
