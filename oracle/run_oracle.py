"""CPU oracle for the device time loop and the built-in initial states.

TEST INFRASTRUCTURE ONLY: restates ``evolve_isothermal`` (jathenax/run.py:20-69),
the problem set-ups (jathenax/run.py:133-163, jathenax/initial_conditions.py:6-15)
and the tanh Kelvin-Helmholtz layer used by the throughput workloads.
"""

from math import isfinite

import numpy as np

from .forcing_oracle import select_update
from .hydro_oracle import primitives, step, timestep


def evolve_iter(U, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim, *, nu=0.0, cs_smag=0.0,
                drag=0.0, forcing=None, dt_update=1.0, t_start=0.0, dedt=0.0, recon="ppm4",
                solver="roe", stress=None, stress_args=None):
    """The loop of ``evolve`` yielding (U, time, dt, cycle) after every cycle; run.py:20-69.

    Reading the state between cycles does not change the run: the sequence of
    yielded states is the trajectory ``evolve`` follows to ``tlim``/``nlim``.
    """
    for name, value in (("viscosity", nu), ("smagorinsky_cs", cs_smag),
                        ("drag_rate", drag), ("dedt", dedt)):
        if not isfinite(value) or value < 0.0:
            raise ValueError(f"{name} must be finite and nonnegative")
    if forcing is not None and (not 0.0 < dt_update < np.inf or not isfinite(t_start)):
        raise ValueError("dt_update must be finite and positive and tdriv_start finite")
    dtype = U.dtype
    time = np.asarray(0.0, dtype=dtype)
    prev = np.asarray(np.inf, dtype=dtype)
    cycle = 0
    update = -1
    raw = np.zeros_like(U[..., 1:3]) if forcing is not None else None
    while time < tlim and cycle < nlim:
        _, W = primitives(U, dfloor)
        dt = np.asarray(timestep(W, dx, dy, cs, cfl, prev, time, tlim,
                                 nu=nu, cs_smag=cs_smag, drag=drag), dtype=dtype)
        power = 0.0
        if forcing is not None:
            table, tables = forcing
            update, raw = select_update(float(time), update, raw, table, tables, dt_update, t_start)
            power = dedt if update >= 0 else 0.0
        U = step(U, dt, dx, dy, cs, dfloor, integrator, nu=nu, cs_smag=cs_smag, drag=drag,
                 raw_force=raw, dedt=power, recon=recon, solver=solver, stress=stress,
                 stress_args=stress_args)
        time = np.asarray(time + dt, dtype=dtype)
        prev = dt
        cycle += 1
        yield U, time, prev, cycle


def evolve(U, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim, **kw):
    """Advance to ``tlim`` or ``nlim`` cycles; returns (U, time, dt, cycle). run.py:20-69.

    Keywords as :func:`evolve_iter` (``forcing`` is ``(table, phase_tables)``).
    Time and dt are kept in U's dtype, as the reference does.
    """
    out = (U, np.asarray(0.0, dtype=U.dtype), np.asarray(np.inf, dtype=U.dtype), 0)
    for out in evolve_iter(U, dx, dy, cs, dfloor, integrator, cfl, tlim, nlim, **kw):
        pass
    return out


def cell_centers(nx, ny):
    """Cell centres on the unit square centred at the origin; run.py:133-135."""
    dx, dy = 1.0 / nx, 1.0 / ny
    return (np.arange(nx) + 0.5) * dx - 0.5, (np.arange(ny) + 0.5) * dy - 0.5


def smooth_state(nx, ny):
    """Smooth periodic density and velocity waves; run.py:159-163."""
    x, y = cell_centers(nx, ny)
    px, py = np.meshgrid(2.0 * np.pi * x, 2.0 * np.pi * y)
    rho = 1.0 + 0.1 * np.sin(px + py)
    vx = 0.2 * np.cos(py)
    vy = 0.2 * np.sin(px)
    return np.stack((rho, rho * vx, rho * vy), axis=-1)


def kh_state(nx, ny):
    """Two shear layers with a cubic-smoothstep tracer; initial_conditions.py:6-15."""
    x, y = cell_centers(nx, ny)
    X, Y = np.meshgrid(x, y)
    dist = np.abs(Y) - 0.25
    ramp = np.clip(-dist / 0.025, -1.0, 1.0)
    s = 0.5 + ramp * (0.75 - 0.25 * ramp**2)
    rho = np.ones_like(s)
    vx = s - 0.5
    vy = 0.02 * np.sin(4 * np.pi * X) * np.exp(-(dist / 0.05)**2)
    return np.stack((rho, rho * vx, rho * vy, rho * s), axis=-1)


def turbulence_state(nx, ny):
    """Unit density at rest; run.py:144."""
    U = np.zeros((ny, nx, 3))
    U[..., 0] = 1.0
    return U
