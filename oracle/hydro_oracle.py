"""CPU oracle for the per-Runge-Kutta-stage isothermal hydro right-hand side.

TEST INFRASTRUCTURE ONLY. This module restates, in NumPy, the algorithm of
JathenAX's ``jathenax/fluxes.py`` and ``jathenax/hydro.py`` (reconstruction,
Riemann solvers, viscous/Smagorinsky stress, SGS stress coupling, flux
divergence, the low-storage RK stages, drag, primitive recovery and the CFL
timestep) so that the CUDA kernels in ``jathenax_gb300`` can be checked
against it. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import it; the shipped package never does.

Every floating-point expression keeps the reference's order of operations, so
that on the same inputs this oracle reproduces the reference run under NumPy
bit for bit (``tests/test_oracle_golden.py`` pins that against fixtures made
from the reference itself by ``tests/golden/make_golden.py``).

Arrays are ``(ny, nx, nvar)``, component innermost: ``(rho, rho*vx, rho*vy,
rho*s1, ...)``. Faces are indexed by the cell on their high-coordinate side:
x-face ``[j, i]`` is the low-x face of cell ``[j, i]``.
"""

import numpy as np

# ---------------------------------------------------------------------------
# Reconstruction: each returns (left, right) primitive states at the low face
# of every cell along ``axis`` (1 = x, 0 = y), with periodic wrap.
# ---------------------------------------------------------------------------


def _nbrs(W, axis):
    """Return W[i-2], W[i-1], W[i+1], W[i+2] along ``axis`` (periodic)."""
    return (np.roll(W, 2, axis=axis), np.roll(W, 1, axis=axis),
            np.roll(W, -1, axis=axis), np.roll(W, -2, axis=axis))


def recon_dc(W, axis):
    """Donor cell; fluxes.py:6-8."""
    return np.roll(W, 1, axis=axis), W


def recon_plm(W, axis):
    """Piecewise linear with the harmonic (van Leer) slope; fluxes.py:11-18."""
    backward = W - np.roll(W, 1, axis=axis)
    forward = np.roll(W, -1, axis=axis) - W
    prod = backward * forward
    same = prod > 0.0
    half_slope = np.where(same, prod / np.where(same, backward + forward, 1.0), 0.0)
    return np.roll(W + half_slope, 1, axis=axis), W - half_slope


def recon_ppm4(W, axis):
    """Fourth-order edge interpolation plus AthenaK's PPM limiter; fluxes.py:21-42."""
    m2, m1, p1, p2 = _nbrs(W, axis)
    lo = (7.0 * (W + m1) - (m2 + p1)) / 12.0
    hi = (7.0 * (W + p1) - (m1 + p2)) / 12.0
    lo = np.fmin(np.fmax(lo, np.fmin(W, m1)), np.fmax(W, m1))
    hi = np.fmin(np.fmax(hi, np.fmin(W, p1)), np.fmax(W, p1))
    d_hi = hi - W
    d_lo = lo - W
    flat = d_hi * d_lo >= 0.0
    lo = np.where(np.abs(d_lo) >= 2.0 * np.abs(d_hi), W - 2.0 * d_hi, lo)
    hi = np.where(np.abs(d_hi) >= 2.0 * np.abs(d_lo), W - 2.0 * d_lo, hi)
    lo = np.where(flat, W, lo)
    hi = np.where(flat, W, hi)
    return np.roll(hi, 1, axis=axis), lo


def _ppmx_limit_edge(a, b, edge, curv_a, curv_b):
    """Smooth-extremum edge limiter for one interface; fluxes.py:45-53."""
    curv = 3.0 * ((a + b) - 2.0 * edge)
    agree = (((curv > 0) & (curv_a > 0) & (curv_b > 0))
             | ((curv < 0) & (curv_a < 0) & (curv_b < 0)))
    smallest = np.fmin(np.abs(curv_a), np.abs(curv_b))
    bounded = np.copysign(np.fmin(1.25 * smallest, np.abs(curv)), curv)
    fixed = 0.5 * (a + b) - np.where(agree, bounded, 0.0) / 6.0
    return np.where((a - edge) * (b - edge) > 0.0, fixed, edge)


def recon_ppmx(W, axis):
    """Extremum-preserving PPM; fluxes.py:56-84."""
    m2, m1, p1, p2 = _nbrs(W, axis)
    lo = (7.0 * (W + m1) - (m2 + p1)) / 12.0
    hi = (7.0 * (W + p1) - (m1 + p2)) / 12.0
    c_left = (m2 + W) - 2.0 * m1
    c_mid = (m1 + p1) - 2.0 * W
    c_right = (W + p2) - 2.0 * p1
    lo = _ppmx_limit_edge(m1, W, lo, c_left, c_mid)
    hi = _ppmx_limit_edge(W, p1, hi, c_mid, c_right)

    d_hi, d_lo = hi - W, lo - W
    extremum = (d_hi * (W - lo) <= 0.0) | ((m1 - W) * (W - p1) <= 0.0)
    curv = 6.0 * (lo + hi - 2.0 * W)
    agree = (((curv > 0) & (c_left > 0) & (c_mid > 0) & (c_right > 0))
             | ((curv < 0) & (c_left < 0) & (c_mid < 0) & (c_right < 0)))
    smallest = np.fmin(np.abs(c_mid), np.fmin(np.abs(c_left), np.abs(c_right)))
    bounded = np.copysign(np.fmin(1.25 * smallest, np.abs(curv)), curv)
    size = np.fmax(np.abs(m1), np.fmax(np.abs(W), np.abs(p1)))
    use = agree & (np.abs(curv) > 1e-12 * size)
    ratio = np.where(use, bounded / np.where(use, curv, 1.0), 0.0)
    lo_mono = np.where(np.abs(d_lo) >= 2.0 * np.abs(d_hi), W - 2.0 * d_hi, lo)
    hi_mono = np.where(np.abs(d_hi) >= 2.0 * np.abs(d_lo), W - 2.0 * d_lo, hi)
    lo = np.where(extremum, W + d_lo * ratio, lo_mono)
    hi = np.where(extremum, W + d_hi * ratio, hi_mono)
    return np.roll(hi, 1, axis=axis), lo


def _wenoz_combine(s0, s1, s2, s3, s4, w0, w1, w2):
    """Weighted sum of the three third-order candidates at one edge; fluxes.py:87-93."""
    a0, a1, a2 = 0.1 * w0, 0.6 * w1, 0.3 * w2
    c0 = 2.0 * s0 - 7.0 * s1 + 11.0 * s2
    c1 = -s1 + 5.0 * s2 + 2.0 * s3
    c2 = 2.0 * s2 + 5.0 * s3 - s4
    return (c0 * a0 + c1 * a1 + c2 * a2) / (6.0 * (a0 + a1 + a2))


def recon_wenoz(W, axis):
    """Fifth-order WENO-Z with rescaled weights; fluxes.py:96-117."""
    m2, m1, p1, p2 = _nbrs(W, axis)
    beta0 = (13.0 / 12.0) * (m2 + W - 2.0 * m1)**2 + 0.25 * (m2 + 3.0 * W - 4.0 * m1)**2
    beta1 = (13.0 / 12.0) * (m1 + p1 - 2.0 * W)**2 + 0.25 * (m1 - p1)**2
    beta2 = (13.0 / 12.0) * (p2 + W - 2.0 * p1)**2 + 0.25 * (p2 + 3.0 * W - 4.0 * p1)**2
    tau5 = np.abs(beta0 - beta2)
    eps = max(1e-42, float(np.finfo(W.dtype).tiny))
    e0, e1, e2 = beta0 + eps, beta1 + eps, beta2 + eps
    emin = np.fmin(e0, np.fmin(e1, e2))
    norm = np.fmax(tau5, emin)
    base = (emin / norm)**2
    ratio = tau5 / norm
    w0 = base + (ratio * (emin / e0))**2
    w1 = base + (ratio * (emin / e1))**2
    w2 = base + (ratio * (emin / e2))**2
    hi = _wenoz_combine(m2, m1, W, p1, p2, w0, w1, w2)
    lo = _wenoz_combine(p2, p1, W, m1, m2, w2, w1, w0)
    return np.roll(hi, 1, axis=axis), lo


RECON = {"dc": recon_dc, "plm": recon_plm, "ppm4": recon_ppm4,
         "ppmx": recon_ppmx, "wenoz": recon_wenoz}


def face_states(W, axis, method, dfloor):
    """Dispatch plus the face density floor for ppmx/wenoz; fluxes.py:126-131."""
    left, right = RECON[method](W, axis)
    if method in ("ppmx", "wenoz"):
        left = left.copy()
        right = right.copy()
        left[..., 0] = np.fmax(left[..., 0], dfloor)
        right[..., 0] = np.fmax(right[..., 0], dfloor)
    return left, right


# ---------------------------------------------------------------------------
# Riemann solvers in the (normal, tangential) frame: return (ny, nx, 3).
# ---------------------------------------------------------------------------


def riemann_roe(dl, dr, ul, ur, tl, tr, cs):
    """Isothermal Roe flux with supersonic upwinding and LLF fallback; fluxes.py:134-172."""
    ml, mr = dl * ul, dr * ur
    ql, qr = dl * tl, dr * tr
    pl, pr = (cs * cs) * dl, (cs * cs) * dr
    f_left = np.stack((ml, ml * ul + pl, ml * tl), axis=-1)
    f_right = np.stack((mr, mr * ur + pr, mr * tr), axis=-1)
    f_mean = 0.5 * (f_left + f_right)

    rl, rr = np.sqrt(dl), np.sqrt(dr)
    inv = 1.0 / (rl + rr)
    u = (rl * ul + rr * ur) * inv
    t = (rl * tl + rr * tr) * inv
    lam_m, lam_p = u - cs, u + cs
    jd, jm, jq = dr - dl, mr - ml, qr - ql
    alpha_m = jd * (0.5 + 0.5 * u / cs) - jm * 0.5 / cs
    alpha_0 = jd * (-t) + jq
    alpha_p = jd * (0.5 - 0.5 * u / cs) + jm * 0.5 / cs
    k_m = -0.5 * np.abs(lam_m) * alpha_m
    k_0 = -0.5 * np.abs(u) * alpha_0
    k_p = -0.5 * np.abs(lam_p) * alpha_p

    flux = np.stack((f_mean[..., 0] + k_m + k_p,
                     f_mean[..., 1] + k_m * lam_m + k_p * lam_p,
                     f_mean[..., 2] + k_m * t + k_0 + k_p * t), axis=-1)
    flux = np.where((lam_m >= 0.0)[..., None], f_left, flux)
    flux = np.where((lam_p <= 0.0)[..., None], f_right, flux)
    d_star = dl + alpha_m
    fallback = (d_star < 0.0) | (d_star + alpha_p < 0.0)
    speed = 0.5 * np.fmax(np.abs(ul) + cs, np.abs(ur) + cs)
    jump = np.stack((jd, jm, jq), axis=-1)
    llf = f_mean - speed[..., None] * jump
    return np.where(fallback[..., None], llf, flux)


def riemann_llf(dl, dr, ul, ur, tl, tr, cs):
    """Local Lax-Friedrichs; fluxes.py:175-183."""
    ml, mr = dl * ul, dr * ur
    ql, qr = dl * tl, dr * tr
    total = np.stack((ml + mr, ml * ul + mr * ur + cs**2 * (dl + dr), ml * tl + mr * tr), axis=-1)
    speed = np.fmax(np.abs(ul) + cs, np.abs(ur) + cs)
    jump = np.stack((dr - dl, mr - ml, qr - ql), axis=-1)
    return 0.5 * (total - speed[..., None] * jump)


def riemann_hlle(dl, dr, ul, ur, tl, tr, cs):
    """HLLE with Roe-averaged wave bounds; fluxes.py:186-201."""
    rl, rr = np.sqrt(dl), np.sqrt(dr)
    u = (rl * ul + rr * ur) * (1.0 / (rl + rr))
    s_lo = np.fmin(u - cs, ul - cs)
    s_hi = np.fmax(u + cs, ur + cs)
    bm = np.where(s_lo < 0.0, s_lo, -1e-20)
    bp = np.where(s_hi > 0.0, s_hi, 1e-20)
    vl, vr = ul - bm, ur - bp
    fl = np.stack((dl * vl, dl * ul * vl + cs**2 * dl, dl * tl * vl), axis=-1)
    fr = np.stack((dr * vr, dr * ur * vr + cs**2 * dr, dr * tr * vr), axis=-1)
    weight = 0.5 * (bp + bm) / (bp - bm)
    return 0.5 * (fl + fr) + weight[..., None] * (fl - fr)


RIEMANN = {"llf": riemann_llf, "hlle": riemann_hlle, "roe": riemann_roe}


def face_flux(left, right, cs, axis, solver="roe"):
    """Gas flux in (x, y) component order plus upwinded scalars; fluxes.py:207-219."""
    n, t = (1, 2) if axis == 1 else (2, 1)
    f = RIEMANN[solver](left[..., 0], right[..., 0], left[..., n], right[..., n],
                        left[..., t], right[..., t], cs)
    if axis == 0:
        f = np.stack((f[..., 0], f[..., 2], f[..., 1]), axis=-1)
    if left.shape[-1] > 3:
        mass = f[..., :1]
        upwind = np.where(mass >= 0, left[..., 3:], right[..., 3:])
        f = np.concatenate((f, mass * upwind), axis=-1)
    return f


# ---------------------------------------------------------------------------
# Viscous and SGS momentum fluxes, divergence.
# ---------------------------------------------------------------------------


def face_gradients(W, dx, dy, axis):
    """(dv/dx, dv/dy) at each low face of ``axis``; fluxes.py:227-238."""
    v = W[..., 1:3]
    d_normal, d_trans = (dx, dy) if axis == 1 else (dy, dx)
    normal = (v - np.roll(v, 1, axis=axis)) / d_normal
    up = np.roll(v, -1, axis=1 - axis)
    down = np.roll(v, 1, axis=1 - axis)
    trans = ((up + np.roll(up, 1, axis=axis))
             - (down + np.roll(down, 1, axis=axis))) / (4.0 * d_trans)
    return (normal, trans) if axis == 1 else (trans, normal)


def eddy_viscosity(grad_x, grad_y, dx, dy, cs_smag):
    """Smagorinsky nu_t = Cs^2 dx dy sqrt(2 S:S); fluxes.py:241-245."""
    shear = grad_x[..., 1] + grad_y[..., 0]
    s2 = 2.0 * (grad_x[..., 0]**2 + grad_y[..., 1]**2) + shear**2
    return cs_smag**2 * dx * dy * np.sqrt(s2)


def viscous_flux(W, dx, dy, nu, cs_smag, axis):
    """Negative viscous stress for the two momentum fluxes; fluxes.py:248-266."""
    gx, gy = face_gradients(W, dx, dy, axis)
    shear = gx[..., 1] + gy[..., 0]
    if axis == 1:
        normal = (4.0 / 3.0) * gx[..., 0] - (2.0 / 3.0) * gy[..., 1]
        stress = np.stack((normal, shear), axis=-1)
    else:
        normal = (4.0 / 3.0) * gy[..., 1] - (2.0 / 3.0) * gx[..., 0]
        stress = np.stack((shear, normal), axis=-1)
    visc = nu
    if cs_smag > 0.0:
        visc = visc + eddy_viscosity(gx, gy, dx, dy, cs_smag)
    rho = W[..., 0]
    mu = 0.5 * visc * (rho + np.roll(rho, 1, axis=axis))
    return -mu[..., None] * stress


def sgs_face_flux(tau):
    """Average cell stresses onto periodic faces; fluxes.py:269-280."""
    if tau.ndim != 3 or tau.shape[-1] != 3:
        raise ValueError("Expected stress with shape (ny, nx, 3)")
    tx, ty = tau[..., :2], tau[..., 1:]
    return 0.5 * (np.roll(tx, 1, axis=1) + tx), 0.5 * (np.roll(ty, 1, axis=0) + ty)


def divergence(fx, fy, dx, dy):
    """Periodic flux divergence; fluxes.py:283-287."""
    return (np.roll(fx, -1, axis=1) - fx) / dx + (np.roll(fy, -1, axis=0) - fy) / dy


# ---------------------------------------------------------------------------
# Time integration (hydro.py).
# ---------------------------------------------------------------------------

# (gamma0, gamma1, beta, delta) per stage; hydro.py:20-36 (AthenaK driver.cpp).
RK_TABLE = {
    "rk2": ((0.0, 1.0, 1.0, None), (0.5, 0.5, 0.5, None)),
    "rk3": ((0.0, 1.0, 1.0, None), (0.25, 0.75, 0.25, None),
            (2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0, None)),
    "rk4": ((0.0, 1.0, 1.193743905974738, None),
            (0.121098479554482, 0.721781678111411, 0.099279895495783, 0.217683334308543),
            (-3.843833699660025, 2.121209265338722, 1.131678018054042, 1.065841341361089),
            (0.546370891121863, 0.198653035682705, 0.310665766509336, 0.0)),
}


def uses_blend_form(gamma0, gamma1):
    """Stages with gamma0 != 0 and gamma0 + gamma1 == 1 use the blend form; hydro.py:46."""
    return gamma0 != 0.0 and gamma0 + gamma1 == 1.0


def rk_combine(U, V, div, dt, coefficients):
    """One low-storage stage on (U, saved register V); hydro.py:39-51."""
    g0, g1, beta, delta = coefficients
    if delta is not None:
        V = V + delta * U
    sdt = beta * dt
    if uses_blend_form(g0, g1):
        return V + (g0 * (U - V) - sdt * div), V
    return g0 * U + g1 * V - sdt * div, V


def primitives(U, dfloor):
    """Floor density in U and return (U, W); hydro.py:54-60."""
    rho = np.where(U[..., 0] < dfloor, dfloor, U[..., 0])
    U = np.concatenate((rho[..., None], U[..., 1:]), axis=-1)
    W = np.concatenate((rho[..., None], (1.0 / rho)[..., None] * U[..., 1:]), axis=-1)
    return U, W


def timestep(W, dx, dy, cs, cfl, prev_dt, time, tlim, *, nu=0.0, cs_smag=0.0, drag=0.0):
    """CFL, diffusion, drag, growth and end-time limits; hydro.py:63-89."""
    limit = np.minimum(np.min(dx / (np.abs(W[..., 1]) + cs)),
                       np.min(dy / (np.abs(W[..., 2]) + cs)))
    if cs_smag > 0.0:
        nu_max = 0.0
        for axis in (0, 1):
            gx, gy = face_gradients(W, dx, dy, axis)
            nu_max = np.maximum(nu_max, np.max(eddy_viscosity(gx, gy, dx, dy, cs_smag)))
        h = min(dx, dy)
        rate = (nu + 2.0 * nu_max) / (h * h)
        with np.errstate(divide="ignore"):
            limit = np.minimum(limit, 0.1875 / rate)
    elif nu > 0.0:
        h = min(dx, dy)
        limit = np.minimum(limit, 0.25 * (h * h) / nu)
    if drag > 0.0:
        limit = np.minimum(limit, 1.0 / drag)
    dt = np.minimum(2.0 * prev_dt, cfl * limit)
    return np.where((time < tlim) & (time + dt > tlim), tlim - time, dt)


def normalized_acceleration(U, raw, dt, dedt):
    """Mean-free acceleration scaled to inject dedt*dt; forcing.py:137-149."""
    rho = U[..., 0, None]
    mom = U[..., 1:3]
    mean = np.sum(rho * raw, axis=(0, 1)) / np.sum(rho)
    f = raw - mean
    f2 = f[..., 0]**2 + f[..., 1]**2
    m0 = np.mean(0.5 * rho[..., 0] * f2 * dt)
    m1 = np.mean(mom[..., 0] * f[..., 0] + mom[..., 1] * f[..., 1])
    with np.errstate(divide="ignore", invalid="ignore"):
        root = np.sqrt(m1 * m1 + 4.0 * m0 * dedt)
        scale = np.where(m1 >= 0.0, 2.0 * dedt / (m1 + root), (root - m1) / (2.0 * m0))
    scale = np.where(m0 > 1e-30, scale, np.nan)
    return np.where(dedt == 0.0, 0.0, scale * f)


def step(U, dt, dx, dy, cs, dfloor, integrator, *, nu=0.0, cs_smag=0.0, drag=0.0,
         raw_force=None, dedt=0.0, recon="ppm4", solver="roe", stress=None,
         stress_args=None, trace=False):
    """One full RK step; hydro.py:92-146.

    ``stress(stress_args, W[..., :3])`` is the optional SGS predictor.
    With ``trace`` the per-stage fields are returned as in hydro.py:135-142.
    """
    U, W = primitives(U, dfloor)
    V = U
    stages = []
    table = RK_TABLE[integrator]
    for number, coeffs in enumerate(table, 1):
        lx, rx = face_states(W, 1, recon, dfloor)
        ly, ry = face_states(W, 0, recon, dfloor)
        fx = face_flux(lx, rx, cs, 1, solver)
        fy = face_flux(ly, ry, cs, 0, solver)
        if nu > 0.0 or cs_smag > 0.0:
            fx = fx.copy()
            fy = fy.copy()
            fx[..., 1:3] = fx[..., 1:3] + viscous_flux(W, dx, dy, nu, cs_smag, 1)
            fy[..., 1:3] = fy[..., 1:3] + viscous_flux(W, dx, dy, nu, cs_smag, 0)
        if stress is not None:
            prim = W[..., :3]
            tau = np.asarray(stress(stress_args, prim))
            if tau.shape != prim.shape or not np.issubdtype(tau.dtype, np.floating):
                raise ValueError("predict_stress must return a floating array of shape (ny, nx, 3)")
            sx, sy = sgs_face_flux(tau.astype(U.dtype))
            fx = fx.copy()
            fy = fy.copy()
            fx[..., 1:3] = fx[..., 1:3] + sx
            fy[..., 1:3] = fy[..., 1:3] + sy
        div = divergence(fx, fy, dx, dy)
        U, V = rk_combine(U, V, div, dt, coeffs)
        if drag > 0.0:
            sdt = coeffs[2] * dt
            U = U.copy()
            U[..., 1:3] = U[..., 1:3] + -((sdt * drag * W[..., 0, None]) * W[..., 1:3])
        kick = raw_force is not None and number == len(table)
        if kick:
            before = U
            accel = normalized_acceleration(U, raw_force, dt, dedt)
            U = U.copy()
            U[..., 1:3] = U[..., 1:3] + U[..., 0, None] * (accel * dt)
        if trace:
            stages.append(dict(primitives=W, left_x=lx, right_x=rx, left_y=ly, right_y=ry,
                               flux_x=fx, flux_y=fy, saved=V, conserved=U))
            if kick:
                stages[-1].update(before_kick=before, acceleration=accel)
        U, W = primitives(U, dfloor)
    if trace:
        return U, tuple(stages)
    return U
