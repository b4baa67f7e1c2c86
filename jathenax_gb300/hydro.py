"""Primitive recovery, Runge-Kutta stages and timestep selection on the GPU.

Drop-in for JathenAX ``jathenax/hydro.py``: same names, arguments, return
values and exceptions. Arrays may be NumPy arrays (copied to the device and
back) or torch CUDA tensors (kept on the device); results come back in the
caller's array type. Every function runs the sm_103a kernels of libjx.so;
there is no CPU path.
"""

import ctypes

import numpy as np

from . import _lib

# Each row is (gam0, gam1, beta, delta), delta None when the stage leaves the
# saved register alone (hydro.py:17-36, AthenaK's low-storage coefficients).
RK_STAGES = {
    "rk2": ((0.0, 1.0, 1.0, None), (0.5, 0.5, 0.5, None)),
    "rk3": ((0.0, 1.0, 1.0, None), (0.25, 0.75, 0.25, None),
            (2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0, None)),
    "rk4": ((0.0, 1.0, 1.193743905974738, None),
            (0.121098479554482, 0.721781678111411, 0.099279895495783, 0.217683334308543),
            (-3.843833699660025, 2.121209265338722, 1.131678018054042, 1.065841341361089),
            (0.546370891121863, 0.198653035682705, 0.310665766509336, 0.0)),
}

TRACE_FIELDS = ("primitives", "left_x", "right_x", "left_y", "right_y", "flux_x", "flux_y",
                "saved", "conserved")


def make_desc(shape, dtype, dx, dy, cs, dfloor, integrator="rk3", *, viscosity=0.0,
              smagorinsky_cs=0.0, drag_rate=0.0, reconstruct="ppm4", rsolver="roe", tile=(0, 0)):
    """Build a jx_desc; unknown selectors raise KeyError like the reference dicts."""
    if len(shape) != 3:
        raise ValueError("state must have shape (ny, nx, nvar)")
    ny, nx, nvar = (int(v) for v in shape)
    desc = _lib.Desc(
        ny=ny, nx=nx, nvar=nvar, dtype=_lib.dtype_id(dtype),
        recon=_lib.RECON_IDS[reconstruct], rsolver=_lib.RSOLVER_IDS[rsolver],
        integrator=_lib.INTEGRATOR_IDS[integrator], tile_x=int(tile[0]), tile_y=int(tile[1]),
        dx=float(dx), dy=float(dy), cs=float(cs), dfloor=float(dfloor),
        viscosity=float(viscosity), smagorinsky_cs=float(smagorinsky_cs),
        drag_rate=float(drag_rate))
    _lib.call("jx_check_desc", ctypes.byref(desc))
    return desc


def rk_stage(U, U_saved, div_flux, dt, coefficients):
    """Apply one AthenaK RK stage to U and the saved register (hydro.py:39-51)."""
    gam0, gam1, beta, delta = coefficients
    Ud = _lib.to_device(U)
    Vd = _lib.to_device(U_saved, Ud.dtype)
    Dd = _lib.to_device(div_flux, Ud.dtype)
    if Vd.shape != Ud.shape or Dd.shape != Ud.shape:
        raise ValueError("U, U_saved and div_flux must have the same shape")
    out = _lib.torch().empty_like(Ud)
    vout = _lib.torch().empty_like(Ud) if delta is not None else None
    _lib.call("jx_rk_stage", _lib.dtype_id(Ud.dtype), Ud.numel(), _lib.ptr(Ud), _lib.ptr(Vd),
              _lib.ptr(Dd), float(dt), float(gam0), float(gam1), float(beta),
              float(delta or 0.0), int(delta is not None), _lib.ptr(out), _lib.ptr(vout),
              _lib.stream_handle())
    saved = vout if delta is not None else Vd
    return _lib.like_input(out, U), _lib.like_input(saved, U)


def recover_isothermal(U, dfloor):
    """Floor density in U and return (U, W) with W = (rho, m/rho, (rho s)/rho) (hydro.py:54-60)."""
    Ud = _lib.to_device(U)
    desc = make_desc(Ud.shape, Ud.dtype, 1.0, 1.0, 1.0, dfloor)
    Uo = _lib.torch().empty_like(Ud)
    W = _lib.torch().empty_like(Ud)
    _lib.call("jx_recover", ctypes.byref(desc), _lib.ptr(Ud), _lib.ptr(Uo), _lib.ptr(W),
              _lib.stream_handle())
    return _lib.like_input(Uo, U), _lib.like_input(W, U)


def _scalar(value):
    if _lib.is_device_array(value):
        return float(value.item())
    return float(value)


def isothermal_timestep(W, dx, dy, cs, cfl, previous_dt, time, tlim, *,
                        viscosity=0.0, smagorinsky_cs=0.0, drag_rate=0.0):
    """AthenaK's hydro, diffusion, drag, growth and end-time limits (hydro.py:63-89)."""
    Wd = _lib.to_device(W)
    desc = make_desc(Wd.shape, Wd.dtype, dx, dy, cs, 1.0, viscosity=viscosity,
                     smagorinsky_cs=smagorinsky_cs, drag_rate=drag_rate)
    ws, nbytes = _lib.workspace(desc)
    out = _lib.torch().empty(1, dtype=_lib.torch().float64, device=_lib.device())
    _lib.call("jx_timestep", ctypes.byref(desc), _lib.ptr(Wd), float(cfl), _scalar(previous_dt),
              _scalar(time), _scalar(tlim), _lib.ptr(out), _lib.ptr(ws), nbytes,
              _lib.stream_handle())
    dt = out.reshape(())
    if _lib.is_device_array(W):
        return dt
    return np.asarray(dt.item(), dtype=np.float64)


class _Forcing:
    """A raw-force buffer (and optionally the OU tables) as a jx_forcing struct."""

    def __init__(self, raw, tables=None):
        self.raw = raw
        self.tables = tables  # (table, cos_x, sin_x, cos_y, sin_y) device tensors
        self.struct = _lib.Forcing(raw_force=raw.data_ptr())
        if tables is not None:
            table, cx, sx, cy, sy = tables
            self.struct.table = table.data_ptr()
            self.struct.cos_x, self.struct.sin_x = cx.data_ptr(), sx.data_ptr()
            self.struct.cos_y, self.struct.sin_y = cy.data_ptr(), sy.data_ptr()
            self.struct.n_updates, self.struct.n_modes = table.shape[0], table.shape[1]


def _trace_buffers(shape, dtype, kick):
    t = _lib.torch()
    bufs = {name: t.empty(shape, dtype=dtype, device=_lib.device()) for name in TRACE_FIELDS}
    if kick:
        bufs["before_kick"] = t.empty(shape, dtype=dtype, device=_lib.device())
        bufs["acceleration"] = t.empty(shape[:2] + (2,), dtype=dtype, device=_lib.device())
    struct = _lib.Trace(**{name: buf.data_ptr() for name, buf in bufs.items()})
    return bufs, struct


def call_predictor(predict_stress, sgs_weights, W, dtype):
    """Run the SGS hook on W[..., :3] and return tau as a contiguous device array.

    The hook receives a torch CUDA tensor of shape (ny, nx, 3) and may return
    any floating array of the same shape (hydro.py:111-119).
    """
    t = _lib.torch()
    primitives = W[..., :3]
    tau = predict_stress(sgs_weights, primitives)
    if not isinstance(tau, t.Tensor):
        tau = t.as_tensor(np.asarray(tau))
    if tuple(tau.shape) != tuple(primitives.shape) or not tau.is_floating_point():
        raise ValueError("predict_stress must return a floating array of shape (ny, nx, 3)")
    return tau.to(device=_lib.device(), dtype=dtype).contiguous()


def run_stages(desc, U_in, *, clock, ws, nbytes, forcing=None, predict_stress=None,
               sgs_weights=None, trace=False, out=None):
    """Enqueue all RK stages of one step reading U_in (not modified).

    Returns (U_out, stages). With ``forcing`` the final stage is followed by
    the normalised kick (clock.power is the effective dedt).
    """
    t = _lib.torch()
    shape = tuple(U_in.shape)
    dtype = U_in.dtype
    schedule = RK_STAGES[_integrator_name(desc.integrator)]
    n = len(schedule)
    stream = _lib.stream_handle()
    scratch = [t.empty_like(U_in), t.empty_like(U_in)]
    final = out if out is not None else t.empty_like(U_in)
    V = U_in
    V_acc = None
    current = U_in
    stages = []
    for number, coefficients in enumerate(schedule, 1):
        last = number == n
        target = final if last else scratch[(number - 1) % 2]
        if coefficients[3] is not None and V_acc is None:
            V_acc = t.empty_like(U_in)
        V_out = V_acc if coefficients[3] is not None else None
        tau = None
        if predict_stress is not None:
            W = t.empty_like(U_in)
            _lib.call("jx_recover", ctypes.byref(desc), _lib.ptr(current), None, _lib.ptr(W), stream)
            tau = call_predictor(predict_stress, sgs_weights, W, dtype)
        kick = forcing is not None and last
        bufs, tstruct = (None, None)
        if trace:
            bufs, tstruct = _trace_buffers(shape, dtype, kick)
        _lib.call("jx_stage", ctypes.byref(desc), number, _lib.ptr(current), _lib.ptr(V),
                  _lib.ptr(target), _lib.ptr(V_out), _lib.ptr(tau), int(kick), _lib.ptr(clock),
                  ctypes.byref(tstruct) if trace else None, _lib.ptr(ws), nbytes, stream)
        if kick:
            _lib.call("jx_force_kick", ctypes.byref(desc), ctypes.byref(forcing.struct),
                      _lib.ptr(target), _lib.ptr(clock),
                      ctypes.byref(tstruct) if trace else None, _lib.ptr(ws), nbytes, stream)
        if trace:
            stages.append(bufs)
        if V_out is not None:
            V = V_acc
        current = target
        # Keep the tau tensor alive until the kernel that reads it is enqueued.
        del tau
    return final, stages


def _integrator_name(code):
    return {v: k for k, v in _lib.INTEGRATOR_IDS.items()}[code]


def isothermal_step(U, dt, dx, dy, cs, dfloor, integrator, *,
                    viscosity=0.0, smagorinsky_cs=0.0, drag_rate=0.0,
                    raw_force=None, dedt=0.0, trace=False, reconstruct="ppm4", rsolver="roe",
                    predict_stress=None, sgs_weights=None):
    """Advance one periodic isothermal step with optional scalar densities (hydro.py:92-146).

    Returns U, or (U, stages) with ``trace`` where each stage is a dict of
    primitives, left_x, right_x, left_y, right_y, flux_x, flux_y, saved and
    conserved (plus before_kick and acceleration on a forced final stage).
    """
    RK_STAGES[integrator]  # KeyError for an unknown integrator, as the reference
    Ud = _lib.to_device(U)
    desc = make_desc(Ud.shape, Ud.dtype, dx, dy, cs, dfloor, integrator, viscosity=viscosity,
                     smagorinsky_cs=smagorinsky_cs, drag_rate=drag_rate,
                     reconstruct=reconstruct, rsolver=rsolver)
    ws, nbytes = _lib.workspace(desc)
    dt_device = _lib.is_device_array(dt)
    clock = _lib.new_clock(dt=0.0 if dt_device else float(dt), power=float(dedt))
    if dt_device:
        clock.view(_lib.torch().float64)[1] = dt.to(_lib.torch().float64).reshape(())
    forcing = None
    if raw_force is not None:
        raw = _lib.to_device(raw_force, Ud.dtype)
        if tuple(raw.shape) != tuple(Ud.shape[:2]) + (2,):
            raise ValueError("raw_force must have shape (ny, nx, 2)")
        forcing = _Forcing(raw)
    final, stages = run_stages(desc, Ud, clock=clock, ws=ws, nbytes=nbytes, forcing=forcing,
                               predict_stress=predict_stress, sgs_weights=sgs_weights, trace=trace)
    result = _lib.like_input(final, U)
    if trace:
        return result, tuple({k: _lib.like_input(v, U) for k, v in s.items()} for s in stages)
    return result


__all__ = ["RK_STAGES", "rk_stage", "recover_isothermal", "isothermal_timestep",
           "isothermal_step", "make_desc", "run_stages"]
