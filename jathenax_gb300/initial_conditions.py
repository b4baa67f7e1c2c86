"""Initial states on the unit square centred at the origin (host NumPy, float64).

``kelvin_helmholtz``, ``smooth_waves`` and ``uniform_rest`` are the reference's
problems (jathenax/initial_conditions.py:6-15, jathenax/run.py:144, 159-163).
``kelvin_helmholtz_tanh`` is the tanh-smoothed shear layer with a tracer used
by the throughput workloads: rho = 1, vx = +-0.5 and s = 1/0 inside/outside
|y| < 0.25 with tanh interfaces of width 0.01, and
vy = 0.01 sin(4 pi x) exp(-(y -+ 0.25)^2 / 0.05^2).
"""

import numpy as np


def cell_centers(nx, ny):
    dx, dy = 1.0 / nx, 1.0 / ny
    return (np.arange(nx) + 0.5) * dx - 0.5, (np.arange(ny) + 0.5) * dy - 0.5


def kelvin_helmholtz(x, y):
    """(rho, rho vx, rho vy, rho s) for two periodic shear layers (initial_conditions.py:6-15)."""
    X, Y = np.meshgrid(x, y)
    gap = np.abs(Y) - 0.25
    t = np.clip(-gap / 0.025, -1.0, 1.0)
    tracer = 0.5 + t * (0.75 - 0.25 * t**2)
    rho = np.ones_like(tracer)
    vx = tracer - 0.5
    vy = 0.02 * np.sin(4 * np.pi * X) * np.exp(-(gap / 0.05)**2)
    return np.stack((rho, rho * vx, rho * vy, rho * tracer), axis=-1)


def kelvin_helmholtz_tanh(nx, ny, width=0.01, amplitude=0.01):
    """Tanh shear layers with a tracer (4 variables)."""
    x, y = cell_centers(nx, ny)
    X, Y = np.meshgrid(x, y)
    inside = 0.5 * (np.tanh((Y + 0.25) / width) - np.tanh((Y - 0.25) / width))
    rho = np.ones_like(X)
    vx = -0.5 + inside
    vy = amplitude * np.sin(4 * np.pi * X) * (np.exp(-((Y - 0.25) / 0.05)**2)
                                              + np.exp(-((Y + 0.25) / 0.05)**2))
    return np.stack((rho, rho * vx, rho * vy, rho * inside), axis=-1)


def smooth_waves(nx, ny):
    """Smooth periodic density and velocity waves (run.py:159-163)."""
    x, y = cell_centers(nx, ny)
    px, py = np.meshgrid(2.0 * np.pi * x, 2.0 * np.pi * y)
    rho = 1.0 + 0.1 * np.sin(px + py)
    vx = 0.2 * np.cos(py)
    vy = 0.2 * np.sin(px)
    return np.stack((rho, rho * vx, rho * vy), axis=-1)


def uniform_rest(nx, ny):
    """Unit density at rest (run.py:144)."""
    U = np.zeros((ny, nx, 3))
    U[..., 0] = 1.0
    return U
