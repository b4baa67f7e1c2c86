"""Turbulence driving: host OU table and GPU render/normalise.

Drop-in for JathenAX ``jathenax/forcing.py``. The host half (random
streams, mode list, OU amplitude table) is exact: integer LCG arithmetic and
IEEE float64 operations in the same order as AthenaK, so the table is bitwise
identical to the reference's. The device half (``render_force``,
``update_force``, ``normalize_force``) runs libjx.so kernels.
"""

import ctypes
from math import log, pi, sqrt

import numpy as np

from . import _lib
from .hydro import _Forcing, make_desc

_M1, _M2 = 2147483563, 2147483399
_A1, _A2 = 40014, 40692
_TOP = 1.0 - np.finfo(float).eps


class _RanSt:
    """AthenaK's RanSt: two LCGs combined through a 32-entry shuffle table."""

    def __init__(self, seed):
        self.s1 = self.s2 = max(1, int(seed))
        self.table = [0] * 32
        for warm in range(40):  # eight discarded draws, then fill slots 31..0
            self.s1 = (_A1 * self.s1) % _M1
            slot = 39 - warm
            if slot < 32:
                self.table[slot] = self.s1
        self.last = self.table[0]
        self.width = 1 + (_M1 - 1) // 32

    def __iter__(self):
        return self

    def __next__(self):
        self.s1 = (_A1 * self.s1) % _M1
        self.s2 = (_A2 * self.s2) % _M2
        slot = self.last // self.width
        self.last = self.table[slot] - self.s2
        self.table[slot] = self.s1
        if self.last < 1:
            self.last += _M1 - 1
        return min((1.0 / _M1) * self.last, _TOP)


def ran_st(seed):
    """Uniform stream in (0, 1) (forcing.py:11-32)."""
    return _RanSt(seed)


def ran_gaussian_st(seed):
    """Polar Box-Muller over ran_st, yielding v2*f then v1*f (forcing.py:35-45)."""
    uniform = _RanSt(seed)
    while True:
        v1 = 2.0 * next(uniform) - 1.0
        v2 = 2.0 * next(uniform) - 1.0
        r2 = v1 * v1 + v2 * v2
        if 0.0 < r2 < 1.0:
            f = sqrt(-2.0 * log(r2) / r2)
            yield v2 * f
            yield v1 * f


def cartesian_modes(nlow, nhigh, kx_bounds, ky_bounds):
    """Signed (kx, ky) with nlow <= |k| <= nhigh, kx outer, ky inner (forcing.py:48-60)."""
    if not 1 <= nlow < nhigh:
        raise ValueError("parabolic driving requires 1 <= nlow < nhigh")
    kx = np.arange(kx_bounds[0], kx_bounds[1] + 1)
    ky = np.arange(ky_bounds[0], ky_bounds[1] + 1)
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    k2 = KX**2 + KY**2
    keep = (k2 >= nlow**2) & (k2 <= nhigh**2)
    modes = np.stack((KX[keep], KY[keep]), axis=-1)
    if len(modes) == 0:
        raise ValueError("no Cartesian forcing modes in the requested band")
    return modes


def modal_coefficients(modes, lengths, nlow, nhigh, npeak, sol_fraction, rseed,
                       tcorr, dt_update, updates):
    """OU modal table [update, mode, dir, re/im] in float64 (forcing.py:63-100).

    Generated by libjx.so's host routine jx_ou_table (C++, integer LCG draws
    and IEEE float64 operations in the reference's order, so the table is
    bitwise the reference's; the tests pin it against the reference's own
    output).
    """
    if not nlow <= npeak <= nhigh or not 0.0 <= sol_fraction <= 1.0:
        raise ValueError("npeak must be in the forcing band and sol_fraction in [0, 1]")
    if not np.isfinite(tcorr) or tcorr < 0.0 or not 0.0 < dt_update < np.inf:
        raise ValueError("tcorr must be finite and nonnegative and dt_update positive")
    modes32 = np.ascontiguousarray(np.asarray(modes), dtype=np.int32)
    out = np.empty((int(updates), len(modes32), 2, 2))
    status = _lib.load().jx_ou_table(
        modes32.ctypes.data_as(ctypes.c_void_p), len(modes32), float(lengths[0]), float(lengths[1]),
        int(nlow), int(nhigh), float(npeak), float(sol_fraction), int(rseed), float(tcorr),
        float(dt_update), int(updates), out.ctypes.data_as(ctypes.c_void_p))
    if status != 0:
        raise ValueError("invalid forcing table arguments")
    return out


def forcing_basis(modes, x, y, lengths, dtype=None):
    """cos/sin(k x) per mode as device arrays [modes, nx] / [modes, ny] (forcing.py:103-108).

    The tables are evaluated in float64 on the host (NumPy's cos/sin, the
    same values the reference obtains under x64) and stored in ``dtype``
    (default: float64).
    """
    modes = np.asarray(_lib.to_device(modes).cpu().numpy() if _lib.is_device_array(modes) else modes)
    x = np.asarray(x.cpu().numpy() if _lib.is_device_array(x) else x, dtype=np.float64)
    y = np.asarray(y.cpu().numpy() if _lib.is_device_array(y) else y, dtype=np.float64)
    k = modes * (2.0 * pi / np.asarray(lengths, dtype=np.float64))
    px = k[:, 0, None] * x
    py = k[:, 1, None] * y
    t = _lib.torch()
    tdtype = t.float64 if dtype is None else dtype
    return tuple(_lib.to_device(a, tdtype) for a in (np.cos(px), np.sin(px), np.cos(py), np.sin(py)))


def _device_tables(coefficients, basis, dtype):
    t = _lib.torch()
    table = _lib.to_device(coefficients, t.float64)
    if table.ndim == 3:
        table = table[None]
    cx, sx, cy, sy = (_lib.to_device(b, dtype) for b in basis)
    if table.ndim != 4 or tuple(table.shape[2:]) != (2, 2):
        raise ValueError("forcing coefficients must have shape (updates, modes, 2, 2)")
    modes = table.shape[1]
    if cx.ndim != 2 or cy.ndim != 2 or cx.shape[0] != modes or cy.shape[0] != modes \
            or sx.shape != cx.shape or sy.shape != cy.shape:
        raise ValueError("forcing basis must be four (modes, nx)/(modes, ny) tables matching "
                         "the coefficient table")
    return table.contiguous(), cx, sx, cy, sy


def render_force(amplitudes, basis, dtype=None):
    """Raw acceleration (ny, nx, 2) summed in AthenaK's mode order (forcing.py:111-122)."""
    t = _lib.torch()
    cx = _lib.to_device(basis[0])
    dtype = dtype or cx.dtype
    tables = _device_tables(amplitudes, basis, dtype)
    nx, ny = tables[1].shape[1], tables[3].shape[1]
    raw = t.empty((ny, nx, 2), dtype=dtype, device=_lib.device())
    forcing = _Forcing(raw, tables)
    desc = make_desc((ny, nx, 3), dtype, 1.0, 1.0, 1.0, 0.0)
    clock = _lib.new_clock(update=0, render=1)
    _lib.call("jx_force_render", ctypes.byref(desc), ctypes.byref(forcing.struct), _lib.ptr(clock),
              _lib.stream_handle())
    return raw if _lib.is_device_array(basis[0]) else raw.cpu().numpy()


def update_force(time, update, raw_force, coefficients, basis, dt_update, tdriv_start):
    """Re-render when the cycle-start time crosses an OU update (forcing.py:125-134)."""
    time = float(time)
    wanted = int(np.floor((time - tdriv_start) / dt_update)) if time >= tdriv_start else -1
    if wanted > int(update):
        table = np.asarray(coefficients.cpu().numpy() if _lib.is_device_array(coefficients)
                           else coefficients)
        row = table[wanted] if 0 <= wanted < len(table) else np.full(table.shape[1:], np.nan)
        raw_force = render_force(row, basis)
    return np.int32(wanted), raw_force


def normalize_force(U, raw_force, dt, dedt):
    """Mean-free acceleration scaled to inject dedt*dt of kinetic energy (forcing.py:137-149)."""
    t = _lib.torch()
    Ud = _lib.to_device(U)
    raw = _lib.to_device(raw_force, Ud.dtype)
    desc = make_desc(Ud.shape, Ud.dtype, 1.0, 1.0, 1.0, 0.0)
    ws, nbytes = _lib.workspace(desc)
    scratch = Ud.clone()
    accel = t.empty(tuple(Ud.shape[:2]) + (2,), dtype=Ud.dtype, device=Ud.device)
    trace = _lib.Trace(acceleration=accel.data_ptr())
    clock = _lib.new_clock(dt=float(dt), power=float(dedt))
    forcing = _Forcing(raw)
    _lib.call("jx_force_kick", ctypes.byref(desc), ctypes.byref(forcing.struct), _lib.ptr(scratch),
              _lib.ptr(clock), ctypes.byref(trace), _lib.ptr(ws), nbytes, _lib.stream_handle())
    return _lib.like_input(accel, U)
