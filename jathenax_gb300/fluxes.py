"""Face operators on the GPU: drop-in for JathenAX ``jathenax/fluxes.py``.

The fused stage kernel (``isothermal_step``) never calls these; they expose
the same reconstruction, Riemann, viscous and SGS-stress operators one at a
time for callers and tests that use them directly. Same names, arguments and
array layouts as the reference; NumPy in gives NumPy out, CUDA tensors stay
on the device.
"""

from functools import partial

from . import _lib


def _face_states(method, W, axis, dfloor=0.0, floor=False):
    Wd = _lib.to_device(W)
    if Wd.ndim == 2:  # (ny, nx) scalar field, as in the reference tests
        out = _face_states(method, Wd[..., None], axis, dfloor, floor)
        left, right = (o[..., 0] for o in out)
        return _lib.like_input(left, W), _lib.like_input(right, W)
    if Wd.ndim != 3:
        raise ValueError("expected W with shape (ny, nx, nvar)")
    if axis not in (0, 1):
        raise ValueError("axis must be 0 (y) or 1 (x)")
    ny, nx, nv = Wd.shape
    left, right = _lib.torch().empty_like(Wd), _lib.torch().empty_like(Wd)
    # Only reconstruct_faces applies the ppmx/wenoz face density floor; the
    # plain *_face_states calls pass NaN, which fmax ignores.
    _lib.call("jx_face_states", _lib.dtype_id(Wd.dtype), _lib.RECON_IDS[method], ny, nx, nv,
              _lib.ptr(Wd), axis, float(dfloor) if floor else float("nan"),
              _lib.ptr(left), _lib.ptr(right), _lib.stream_handle())
    return _lib.like_input(left, W), _lib.like_input(right, W)


def dc_face_states(W, axis):
    """Donor cell: the two adjacent cell averages (fluxes.py:6-8)."""
    return _face_states("dc", W, axis)


def plm_face_states(W, axis):
    """Piecewise linear with AthenaK's harmonic limiter (fluxes.py:11-18)."""
    return _face_states("plm", W, axis)


def ppm4_face_states(W, axis):
    """Fourth-order PPM edges with AthenaK's limiter (fluxes.py:21-42)."""
    return _face_states("ppm4", W, axis)


def ppmx_face_states(W, axis):
    """Extremum-preserving PPM (fluxes.py:56-84)."""
    return _face_states("ppmx", W, axis)


def wenoz_face_states(W, axis):
    """Fifth-order WENO-Z (fluxes.py:96-117)."""
    return _face_states("wenoz", W, axis)


RECONSTRUCTIONS = {
    "dc": dc_face_states, "plm": plm_face_states, "ppm4": ppm4_face_states,
    "ppmx": ppmx_face_states, "wenoz": wenoz_face_states,
}


def reconstruct_faces(W, axis, reconstruct, dfloor):
    """Dispatch plus the ppmx/wenoz face density floor (fluxes.py:126-131)."""
    RECONSTRUCTIONS[reconstruct]  # KeyError for unknown names
    return _face_states(reconstruct, W, axis, dfloor, floor=reconstruct in ("ppmx", "wenoz"))


def isothermal_flux(left, right, cs, axis, rsolver="roe"):
    """Gas and passive-scalar fluxes in x/y component order (fluxes.py:207-219)."""
    code = _lib.RSOLVER_IDS[rsolver]
    L = _lib.to_device(left)
    R = _lib.to_device(right, L.dtype)
    if L.shape != R.shape or L.shape[-1] < 3:
        raise ValueError("left and right must share a shape (..., nvar >= 3)")
    if axis not in (0, 1):
        raise ValueError("axis must be 0 (y) or 1 (x)")
    flux = _lib.torch().empty_like(L)
    nv = L.shape[-1]
    _lib.call("jx_face_flux", _lib.dtype_id(L.dtype), code, L.numel() // nv, nv, axis,
              _lib.ptr(L), _lib.ptr(R), float(cs), _lib.ptr(flux), _lib.stream_handle())
    return _lib.like_input(flux, left)


def roe_isothermal_flux(left, right, cs, axis):
    """AthenaK's isothermal Roe flux, including any passive scalars (fluxes.py:222-224)."""
    return isothermal_flux(left, right, cs, axis)


def _solver(name, rho_l, rho_r, vn_l, vn_r, vt_l, vt_r, cs):
    """Riemann solver in the (normal, tangential) frame; returns (..., 3)."""
    t = _lib.torch()
    parts = [_lib.to_device(a) for a in (rho_l, vn_l, vt_l, rho_r, vn_r, vt_r)]
    dtype = parts[0].dtype
    parts = [p.to(dtype) for p in parts]
    left = t.stack(parts[:3], dim=-1).contiguous()
    right = t.stack(parts[3:], dim=-1).contiguous()
    flux = isothermal_flux(left, right, cs, 1, name)
    return _lib.like_input(flux, rho_l)


RIEMANN_SOLVERS = {name: partial(_solver, name) for name in ("llf", "hlle", "roe")}


def face_velocity_gradients(W, dx, dy, axis):
    """(dv/dx, dv/dy) of both velocity components at each low face along axis (fluxes.py:227-238)."""
    Wd = _lib.to_device(W)
    if Wd.ndim != 3 or Wd.shape[-1] < 3:
        raise ValueError("expected W with shape (ny, nx, nvar >= 3)")
    ny, nx, nv = Wd.shape
    t = _lib.torch()
    gx = t.empty((ny, nx, 2), dtype=Wd.dtype, device=Wd.device)
    gy = t.empty((ny, nx, 2), dtype=Wd.dtype, device=Wd.device)
    _lib.call("jx_face_velocity_gradients", _lib.dtype_id(Wd.dtype), ny, nx, nv, _lib.ptr(Wd), float(dx), float(dy),
              int(axis), _lib.ptr(gx), _lib.ptr(gy), _lib.stream_handle())
    return _lib.like_input(gx, W), _lib.like_input(gy, W)


def smagorinsky_viscosity(dv_dx, dv_dy, dx, dy, smagorinsky_cs):
    """Kinematic eddy viscosity (Cs sqrt(dx dy))^2 times the strain norm (fluxes.py:241-245)."""
    gx = _lib.to_device(dv_dx)
    gy = _lib.to_device(dv_dy, gx.dtype)
    if gx.shape != gy.shape or gx.ndim != 3 or gx.shape[-1] != 2:
        raise ValueError("expected two gradient arrays of shape (ny, nx, 2)")
    out = _lib.torch().empty(tuple(gx.shape[:2]), dtype=gx.dtype, device=gx.device)
    _lib.call("jx_smagorinsky_viscosity", _lib.dtype_id(gx.dtype), gx.shape[0] * gx.shape[1], _lib.ptr(gx),
              _lib.ptr(gy), float(dx), float(dy), float(smagorinsky_cs), _lib.ptr(out), _lib.stream_handle())
    return _lib.like_input(out, dv_dx)


def viscous_momentum_flux(W, dx, dy, viscosity, smagorinsky_cs, axis):
    """Negative viscous (plus Smagorinsky) stress for the momentum fluxes (fluxes.py:248-266)."""
    Wd = _lib.to_device(W)
    if Wd.ndim != 3 or Wd.shape[-1] < 3:
        raise ValueError("expected W with shape (ny, nx, nvar >= 3)")
    ny, nx, nv = Wd.shape
    out = _lib.torch().empty((ny, nx, 2), dtype=Wd.dtype, device=Wd.device)
    _lib.call("jx_viscous_flux", _lib.dtype_id(Wd.dtype), ny, nx, nv, _lib.ptr(Wd), float(dx),
              float(dy), float(viscosity), float(smagorinsky_cs), axis, _lib.ptr(out),
              _lib.stream_handle())
    return _lib.like_input(out, W)


def stress_face_fluxes(tau):
    """Cell-centred (tau_xx, tau_xy, tau_yy) to periodic face momentum fluxes (fluxes.py:269-280)."""
    shape = tuple(getattr(tau, "shape", ()))
    if len(shape) != 3 or shape[-1] != 3:
        raise ValueError("Expected stress with shape (ny, nx, 3)")
    T = _lib.to_device(tau)
    ny, nx, _ = T.shape
    fx = _lib.torch().empty((ny, nx, 2), dtype=T.dtype, device=T.device)
    fy = _lib.torch().empty((ny, nx, 2), dtype=T.dtype, device=T.device)
    _lib.call("jx_stress_face_fluxes", _lib.dtype_id(T.dtype), ny, nx, _lib.ptr(T), _lib.ptr(fx),
              _lib.ptr(fy), _lib.stream_handle())
    return _lib.like_input(fx, tau), _lib.like_input(fy, tau)


def flux_divergence(flux_x, flux_y, dx, dy):
    """Difference the high and low faces of each periodic cell (fluxes.py:283-287)."""
    Fx = _lib.to_device(flux_x)
    Fy = _lib.to_device(flux_y, Fx.dtype)
    if Fx.shape != Fy.shape or Fx.ndim != 3:
        raise ValueError("flux_x and flux_y must share a shape (ny, nx, nv)")
    ny, nx, nv = Fx.shape
    div = _lib.torch().empty_like(Fx)
    _lib.call("jx_flux_divergence", _lib.dtype_id(Fx.dtype), ny, nx, nv, _lib.ptr(Fx), _lib.ptr(Fy),
              float(dx), float(dy), _lib.ptr(div), _lib.stream_handle())
    return _lib.like_input(div, flux_x)

