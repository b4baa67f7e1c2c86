"""CPU oracle for the turbulence driver (host RNG, OU table, force rendering).

TEST INFRASTRUCTURE ONLY: restates JathenAX ``jathenax/forcing.py`` in NumPy
and plain Python so the GPU render/normalise kernels and the package's own
host-side table builder can be checked against it. The uniform and Gaussian
streams are exact integer/IEEE restatements (bit-identical by construction).
"""

from fractions import Fraction
from math import exp, log, pi, sqrt

import numpy as np


def uniform_stream(seed):
    """Shuffled two-LCG uniform generator (AthenaK RanSt); forcing.py:11-32."""
    m1, m2 = 2147483563, 2147483399
    s1 = s2 = max(1, seed)
    table = [0] * 32
    for slot in range(39, -1, -1):
        s1 = (40014 * s1) % m1
        if slot < 32:
            table[slot] = s1
    last = table[0]
    width = 1 + (m1 - 1) // 32
    top = 1.0 - np.finfo(float).eps
    while True:
        s1 = (40014 * s1) % m1
        s2 = (40692 * s2) % m2
        slot = last // width
        last = table[slot] - s2
        table[slot] = s1
        if last < 1:
            last += m1 - 1
        yield min((1.0 / m1) * last, top)


def gaussian_stream(seed):
    """Polar Box-Muller returning v2*scale then v1*scale; forcing.py:35-45."""
    u = uniform_stream(seed)
    while True:
        a = 2.0 * next(u) - 1.0
        b = 2.0 * next(u) - 1.0
        r2 = a * a + b * b
        if 0.0 < r2 < 1.0:
            f = sqrt(-2.0 * log(r2) / r2)
            yield b * f
            yield a * f


def forcing_modes(nlow, nhigh, kx_range, ky_range):
    """Signed integer modes in the band, kx outer and ky inner; forcing.py:48-60."""
    if not 1 <= nlow < nhigh:
        raise ValueError("parabolic driving requires 1 <= nlow < nhigh")
    out = []
    for kx in range(kx_range[0], kx_range[1] + 1):
        for ky in range(ky_range[0], ky_range[1] + 1):
            if nlow**2 <= kx**2 + ky**2 <= nhigh**2:
                out.append((kx, ky))
    if not out:
        raise ValueError("no Cartesian forcing modes in the requested band")
    return np.asarray(out)


def _fma(a, b, c):
    """Correctly rounded a*b + c through exact rational arithmetic."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def ou_table(modes, lengths, nlow, nhigh, npeak, sol_fraction, seed, tcorr, dt_update, updates):
    """OU modal amplitudes [update, mode, dir, re/im] in float64; forcing.py:63-100."""
    if not nlow <= npeak <= nhigh or not 0.0 <= sol_fraction <= 1.0:
        raise ValueError("npeak must be in the forcing band and sol_fraction in [0, 1]")
    if not np.isfinite(tcorr) or tcorr < 0.0 or not 0.0 < dt_update < np.inf:
        raise ValueError("tcorr must be finite and nonnegative and dt_update positive")
    dk = 2.0 * pi / np.asarray(lengths)
    k = modes * dk
    kmag = np.sqrt(k[:, 0]**2 + k[:, 1]**2)
    kpeak = npeak * 2.0 * pi / lengths[0]
    band = nhigh * max(dk) - nlow * min(dk)
    slope = float(-4.0 / band**2)
    power = np.asarray([_fma(slope, float(d2), 1.0) for d2 in (kmag - kpeak)**2])
    amp = np.sqrt(np.abs(power))
    amp *= np.sqrt(kpeak / kmag)

    corr = exp(-dt_update / tcorr) if tcorr > 1e-6 else 0.0
    kick = sqrt(1.0 - corr * corr)
    draws = gaussian_stream(seed)
    table = np.empty((updates, len(modes), 2, 2))
    for u in range(updates):
        noise = np.fromiter(draws, dtype=float, count=4 * len(modes)).reshape(-1, 2, 2)
        noise *= amp[:, None, None]
        kn = k[:, 0, None] * noise[:, 0] + k[:, 1, None] * noise[:, 1]
        along = k[:, :, None] * kn[:, None] / kmag[:, None, None]**2
        noise = sol_fraction * (noise - along) + (1.0 - sol_fraction) * along
        table[u] = noise if u == 0 else corr * table[u - 1] + kick * noise
    return table


def phase_tables(modes, x, y, lengths):
    """cos/sin of k.x per mode along each axis; forcing.py:103-108."""
    k = modes * (2.0 * pi / np.asarray(lengths, dtype=x.dtype))
    px = k[:, 0, None] * x
    py = k[:, 1, None] * y
    return np.cos(px), np.sin(px), np.cos(py), np.sin(py)


def render(amplitudes, tables):
    """Raw acceleration (ny, nx, 2), summed in mode order; forcing.py:111-122."""
    cx, sx, cy, sy = tables
    force = np.zeros((cy.shape[1], cx.shape[1], 2), amplitudes.dtype)
    for n in range(len(amplitudes)):
        re = cx[n] * cy[n, :, None] - sx[n] * sy[n, :, None]
        im = cx[n] * sy[n, :, None] + sx[n] * cy[n, :, None]
        force = force + (re[..., None] * amplitudes[n, :, 0] - im[..., None] * amplitudes[n, :, 1])
    return force


def select_update(time, update, raw, table, tables, dt_update, t_start):
    """Re-render when the cycle-start time crosses an OU update; forcing.py:125-134."""
    wanted = int(np.floor((time - t_start) / dt_update)) if time >= t_start else -1
    if wanted > update:
        amplitudes = table[wanted] if 0 <= wanted < len(table) else np.full(table.shape[1:], np.nan)
        raw = render(amplitudes, tables)
    return wanted, raw
