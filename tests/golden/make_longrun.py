"""Generate ``longrun.npz``: whole-run float64 oracle trajectories of the stated
throughput configurations, with their chaos floors.

Usage:

    python tests/golden/make_longrun.py [--reference <path-to-JathenAX-checkout>] [--jobs N]

Cases (the oracle, ``oracle/run_oracle.evolve_iter``, which
``tests/test_oracle_golden.py`` pins bit for bit to the reference's own runs):

* the tanh Kelvin-Helmholtz layer with a tracer on 128 x 128 cells (width
  0.01, vy amplitude 0.01, 4 variables), CFL 0.4, run to t = 3, for
  ppm4/roe/rk3, wenoz/hlle/rk2, ppmx/llf/rk4, plm/hlle/rk3 and dc/llf/rk2;
* the driven-turbulence deck on 128 x 128 cells (seed 1618, 56 modes,
  nu 1.5e-6, drag 0.3333335, dedt 0.03703705, rk3/ppm4/roe) for 300 cycles.

For each case the fixture holds the initial state (``kh_U0``, ``turb_U0``),
the oracle's state at a few snapshot cycles (the state after that cycle of the uninterrupted run) and
the time reached there, and two chaos floors: the same run started from the
density multiplied by 1 + eps * noise (seeded Gaussian noise, eps = 1e-12 and
1e-15), compared with the unperturbed run every 25 cycles (largest error
over the grid, per component, relative to that component's largest
magnitude). A float64 implementation whose rounding differs from NumPy's (FMA
contraction, reciprocals) cannot be expected to stay closer to the oracle
than these floors once they exceed the parity tolerance.

With ``--reference`` the reference's own ``evolve_isothermal`` is also run
under ``oracle/jaxshim`` for the ppm4/roe/rk3 case to t = 3, and the script
stops unless its final state equals the oracle's bit for bit.

Nothing at test time reads the reference tree or reruns these trajectories.
"""

import argparse
import multiprocessing as mp
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
SHIM = REPO / "oracle" / "jaxshim"
N = 128
TLIM = 3.0
EPSILONS = (1e-12, 1e-15)
FLOOR_EVERY = 25

# case -> (problem, reconstruct, rsolver, integrator, snapshot spec)
# A snapshot spec entry is ("c", cycle) or ("t", time): the first cycle whose
# end time reaches it; the last cycle of the run is always a snapshot.
CASES = {
    "kh_ppm4_roe_rk3": ("kh", "ppm4", "roe", "rk3", (("c", 25), ("t", 1.0), ("t", 2.0))),
    "kh_wenoz_hlle_rk2": ("kh", "wenoz", "hlle", "rk2", (("c", 1), ("c", 25), ("t", 1.0), ("t", 2.2))),
    "kh_ppmx_llf_rk4": ("kh", "ppmx", "llf", "rk4", (("c", 1), ("t", 1.0))),
    "kh_plm_hlle_rk3": ("kh", "plm", "hlle", "rk3", ()),
    "kh_dc_llf_rk2": ("kh", "dc", "llf", "rk2", ()),
    "turb_ppm4_roe_rk3": ("turbulence", "ppm4", "roe", "rk3", ()),
}
# With --dense (a larger fixture for tabulating errors against time, not
# committed): more snapshots of the same trajectories.
DENSE_EXTRA = {
    "kh_ppm4_roe_rk3": (("t", 0.5), ("t", 1.5), ("t", 2.5)),
    "kh_ppmx_llf_rk4": (("c", 25),),
    "kh_plm_hlle_rk3": (("t", 1.0),),
    "kh_dc_llf_rk2": (("t", 1.0),),
    "turb_ppm4_roe_rk3": (("c", 100),),
}
TURB_CYCLES = 300


def initial_state(problem):
    sys.path.insert(0, str(REPO))
    from jathenax_gb300.initial_conditions import kelvin_helmholtz_tanh, uniform_rest
    return kelvin_helmholtz_tanh(N, N) if problem == "kh" else uniform_rest(N, N)


def turbulence_forcing():
    """OU table (seed 1618, enough updates for the run) and phase tables."""
    sys.path.insert(0, str(REPO))
    from oracle import forcing_oracle as F
    from oracle.run_oracle import cell_centers
    modes = F.forcing_modes(3, 5, (-5, 5), (-5, 5))
    table = F.ou_table(modes, (1.0, 1.0), 3, 5, 4.0, 1.0, 1618, 0.75, 0.0075, 200)
    x, y = cell_centers(N, N)
    return table, F.phase_tables(modes, x, y, (1.0, 1.0))


def run_kwargs(problem, recon, solver, forcing):
    kw = dict(recon=recon, solver=solver)
    if problem == "turbulence":
        kw.update(nu=1.5e-6, drag=0.3333335, forcing=forcing, dt_update=0.0075, t_start=0.0, dedt=0.03703705)
    return kw


def trajectory(job):
    """Run one case (eps = 0: the oracle; else the perturbed run); return its
    states every FLOOR_EVERY cycles, at the snapshot cycles and at the end."""
    name, eps, U0, forcing, dense = job
    sys.path.insert(0, str(REPO))
    from oracle.run_oracle import evolve_iter
    problem, recon, solver, integ, spec = CASES[name]
    if dense:
        spec = spec + DENSE_EXTRA.get(name, ())
    U = U0.copy()
    if eps:
        noise = np.random.default_rng(45).standard_normal(U.shape[:2])
        U[..., 0] *= 1.0 + eps * noise
    dfloor = 1.17549e-38 if problem == "turbulence" else 1e-10
    tlim, nlim = (1e30, TURB_CYCLES) if problem == "turbulence" else (TLIM, 10**7)
    wanted_t = sorted(v for k, v in spec if k == "t")
    wanted_c = {v for k, v in spec if k == "c"}
    out = {}
    snaps = []
    for Un, time, _, cycle in evolve_iter(U, 1.0 / N, 1.0 / N, 1.0, dfloor, integ, 0.4, tlim, nlim,
                                          **run_kwargs(problem, recon, solver, forcing)):
        if cycle % FLOOR_EVERY == 0:
            out[cycle] = (float(time), Un)
        hit = cycle in wanted_c
        while wanted_t and float(time) >= wanted_t[0]:
            wanted_t.pop(0)
            hit = True
        if hit:
            snaps.append(cycle)
            out[cycle] = (float(time), Un)
    out[cycle] = (float(time), Un)
    snaps.append(cycle)
    return name, eps, out, sorted(set(snaps))


def max_rel(a, b):
    a2, b2 = a.reshape(-1, a.shape[-1]), b.reshape(-1, b.shape[-1])
    scale = np.maximum(np.max(np.abs(b2), axis=0), 1e-300)
    return np.max(np.abs(a2 - b2), axis=0) / scale


def reference_final(reference, U0):
    """The reference's evolve_isothermal under the shim, ppm4/roe/rk3 to t=3."""
    sys.path[:0] = [str(SHIM), str(reference)]
    import jax.numpy as jnp
    from jathenax import run
    out = run.evolve_isothermal(jnp.asarray(U0), 1.0 / N, 1.0 / N, 1.0, 1e-10, "rk3", 0.4, TLIM, 10**7)
    return np.asarray(out[0]), float(out[1]), int(out[3])


def main():
    parser = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    parser.add_argument("--reference", type=Path, default=None)
    parser.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    parser.add_argument("--dense", action="store_true", help="also the DENSE_EXTRA snapshots (writes longrun_dense.npz)")
    args = parser.parse_args()
    forcing = turbulence_forcing()
    starts = {name: initial_state(CASES[name][0]) for name in CASES}
    jobs = [(name, eps, starts[name], forcing if CASES[name][0] == "turbulence" else None, args.dense)
            for name in CASES for eps in (0.0,) + EPSILONS]
    # spawn: workers start clean (no inherited threads or device state).
    with mp.get_context("spawn").Pool(min(args.jobs, len(jobs))) as pool:
        results = pool.map(trajectory, jobs)
    runs = {(name, eps): (out, snaps) for name, eps, out, snaps in results}

    fixture = {"n": np.int32(N), "tlim": np.float64(TLIM), "floor_eps": np.asarray(EPSILONS),
               "turb_table": forcing[0], "turb_cos_x": forcing[1][0], "turb_sin_x": forcing[1][1],
               "turb_cos_y": forcing[1][2], "turb_sin_y": forcing[1][3],
               "kh_U0": starts["kh_ppm4_roe_rk3"], "turb_U0": starts["turb_ppm4_roe_rk3"]}
    for name in CASES:
        base, snaps = runs[(name, 0.0)]
        fixture[f"{name}_snap_cycles"] = np.asarray(snaps, dtype=np.int32)
        fixture[f"{name}_snap_times"] = np.asarray([base[c][0] for c in snaps])
        for c in snaps:
            fixture[f"{name}_U_{c}"] = base[c][1]
        for eps in EPSILONS:
            pert, _ = runs[(name, eps)]
            cycles = sorted(c for c in base if c in pert)
            fixture[f"{name}_floor_{eps:.0e}_cycles"] = np.asarray(cycles, dtype=np.int32)
            fixture[f"{name}_floor_{eps:.0e}_times"] = np.asarray([base[c][0] for c in cycles])
            fixture[f"{name}_floor_{eps:.0e}_err"] = np.asarray([max_rel(pert[c][1], base[c][1]) for c in cycles])
        print(name, "snapshots", snaps, "times", np.round(fixture[f"{name}_snap_times"], 4), flush=True)
        for eps in EPSILONS:
            err = fixture[f"{name}_floor_{eps:.0e}_err"].max(axis=1)
            print(f"   floor {eps:.0e}: end {err[-1]:.2e}, max {err.max():.2e}", flush=True)

    if args.reference is not None:
        ref_U, ref_t, ref_c = reference_final(args.reference.resolve(), starts["kh_ppm4_roe_rk3"])
        name = "kh_ppm4_roe_rk3"
        last = int(fixture[f"{name}_snap_cycles"][-1])
        mine = fixture[f"{name}_U_{last}"]
        if ref_c != last or not np.array_equal(ref_U.view(np.uint64), mine.view(np.uint64)):
            sys.exit(f"oracle and reference differ at t=3 (cycles {last} vs {ref_c})")
        fixture["meta_reference_check"] = np.asarray(f"{name}: oracle final state equals the reference's "
                                                     f"evolve_isothermal under the shim bit for bit "
                                                     f"({ref_c} cycles, t={ref_t})")
        print("reference check:", str(fixture["meta_reference_check"]))
    path = HERE / ("longrun_dense.npz" if args.dense else "longrun.npz")
    np.savez_compressed(path, **fixture)
    print("wrote", path, f"{path.stat().st_size / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
