// The fused RK-stage kernel: one CTA owns a TX x TY tile of cells.
//
//   phase 0  load the tile plus a periodic ghost halo of depth H from U,
//            floor rho and convert to primitives W in shared memory
//            (recover_isothermal, hydro.py:54-60);
//   phase 1  reconstruct low/high edge values of every cell needed by the
//            tile's x- and y-faces (fluxes.py:6-131) into face-left/right
//            arrays in shared memory;
//   phase 2  Riemann-solve every face (fluxes.py:134-219), add the viscous /
//            Smagorinsky stress (fluxes.py:227-266) and the SGS stress
//            (fluxes.py:269-280) and overwrite the left state with the flux;
//   phase 3  flux divergence (fluxes.py:283-287), RK combine
//            (hydro.py:39-51), drag (hydro.py:122-125), density floor
//            (hydro.py:143) and the write-back, plus the CFL partial max of
//            the new state (hydro.py:66-68) on the last stage.
//
// Each face state is reconstructed once per cell (both edges from one
// 5-point stencil), each flux is solved once per face, and nothing but the
// stage output (and the RK4 saved register) goes back to HBM.
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"

namespace jx {

template <typename R, int RECON, int RS>
__global__ void __launch_bounds__(kStageThreads) stage_kernel(const StageParams p) {
  if (p.clock->done) return;
  constexpr int H = TileHalo<RECON>::value;
  constexpr bool kFaceFloor = RECON == JX_PPMX || RECON == JX_WENOZ;  // fluxes.py:128-130
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32 * 2];

  const int tid = threadIdx.x;
  const int NV = p.nv, TX = p.tx, TY = p.ty;
  const int bx = blockIdx.x % p.tiles_x, by = blockIdx.x / p.tiles_x;
  const int x0 = bx * TX, y0 = by * TY;
  const int tw = min(TX, p.nx - x0), th = min(TY, p.ny - y0);
  const int PW = TX + 2 * H, PH = TY + 2 * H;
  const int wplane = PW * PH;
  const int fxp = TX + 1;               // x-face row pitch
  const int fxplane = TY * fxp;
  const int fyplane = (TY + 1) * TX;    // y-face row pitch is TX
  R* sW = reinterpret_cast<R*>(smem_raw);
  R* sLx = sW + NV * wplane;
  R* sRx = sLx + NV * fxplane;
  R* sLy = sRx + NV * fxplane;
  R* sRy = sLy + NV * fyplane;

  const R* __restrict__ U = static_cast<const R*>(p.U);
  const R dfloor = static_cast<R>(p.dfloor);

  // ---- phase 0: halo load + primitive recovery --------------------------
  const int lw = tw + 2 * H, lh = th + 2 * H;
  for (int idx = tid; idx < lw * lh; idx += kStageThreads) {
    const int ly = idx / lw, lx = idx - ly * lw;
    const int gy = wrap_index(y0 + ly - H, p.ny), gx = wrap_index(x0 + lx - H, p.nx);
    const R* u = U + ((size_t)gy * p.nx + gx) * NV;
    R rho = u[0];
    rho = rho < dfloor ? dfloor : rho;
    const R inv = R(1) / rho;
    const int s = ly * PW + lx;
    sW[s] = rho;
    for (int v = 1; v < NV; ++v) sW[v * wplane + s] = inv * u[v];
  }
  __syncthreads();

  // ---- phase 1: edge reconstruction ---------------------------------------
  {
    const int nxr = th * (tw + 2);   // rows 0..th-1, cells -1..tw
    const int nyr = (th + 2) * tw;   // rows -1..th, columns 0..tw-1
    for (int idx = tid; idx < nxr + nyr; idx += kStageThreads) {
      const bool xs = idx < nxr;
      int r, c, stride;
      if (xs) {
        r = idx / (tw + 2);
        c = idx - r * (tw + 2) - 1;
        stride = 1;
      } else {
        const int k = idx - nxr;
        r = k / tw - 1;
        c = k - (r + 1) * tw;
        stride = PW;
      }
      const int s = (r + H) * PW + (c + H);
      for (int v = 0; v < NV; ++v) {
        const R* w = sW + v * wplane + s;
        const R q0 = w[0];
        const R qm1 = H >= 2 ? w[-stride] : q0;
        const R qp1 = H >= 2 ? w[stride] : q0;
        const R qm2 = H >= 3 ? w[-2 * stride] : q0;
        const R qp2 = H >= 3 ? w[2 * stride] : q0;
        R lo, hi;
        edges<RECON>(qm2, qm1, q0, qp1, qp2, lo, hi);
        if (kFaceFloor && v == 0) {
          lo = fmax(lo, dfloor);
          hi = fmax(hi, dfloor);
        }
        if (xs) {
          if (c + 1 <= tw) sLx[v * fxplane + r * fxp + c + 1] = hi;
          if (c >= 0) sRx[v * fxplane + r * fxp + c] = lo;
        } else {
          if (r + 1 <= th) sLy[v * fyplane + (r + 1) * TX + c] = hi;
          if (r >= 0) sRy[v * fyplane + r * TX + c] = lo;
        }
      }
    }
  }
  __syncthreads();

  // ---- phase 2: Riemann solve + viscous + SGS stress ----------------------
  {
    Gas<R> gas;
    gas.cs = static_cast<R>(p.cs);
    gas.cs2 = static_cast<R>(p.cs * p.cs);
    gas.inv_cs = static_cast<R>(1.0 / p.cs);
    gas.half_inv_cs = static_cast<R>(0.5 / p.cs);
    const R* __restrict__ tau = static_cast<const R*>(p.tau);
    const int nfx = th * (tw + 1), nfy = (th + 1) * tw;
    for (int idx = tid; idx < nfx + nfy; idx += kStageThreads) {
      const bool xs = idx < nfx;
      int r, c, fo, fplane;
      R* L;
      R* Rt;
      if (xs) {
        r = idx / (tw + 1);
        c = idx - r * (tw + 1);
        fo = r * fxp + c;
        fplane = fxplane;
        L = sLx;
        Rt = sRx;
      } else {
        const int k = idx - nfx;
        r = k / tw;
        c = k - r * tw;
        fo = r * TX + c;
        fplane = fyplane;
        L = sLy;
        Rt = sRy;
      }
      const int nn = xs ? 1 : 2, tt = xs ? 2 : 1;
      const R dl = L[fo], dr = Rt[fo];
      const R nl = L[nn * fplane + fo], nr = Rt[nn * fplane + fo];
      const R tl = L[tt * fplane + fo], tr = Rt[tt * fplane + fo];
      R f0, fn, ft;
      riemann<RS>(dl, dr, nl, nr, tl, tr, gas, f0, fn, ft);
      R f1 = xs ? fn : ft;
      R f2 = xs ? ft : fn;

      if (p.visc_on) {
        // Cell b is on the high side of the face, cell a on the low side.
        const int sb = (r + H) * PW + (c + H);
        const int sa = xs ? sb - 1 : sb - PW;
        const R* vx = sW + wplane;
        const R* vy = sW + 2 * wplane;
        R dvx_dx, dvy_dx, dvx_dy, dvy_dy;
        if (xs) {
          const R inv_n = static_cast<R>(p.inv_dx), inv_t = static_cast<R>(p.inv_4dy);
          dvx_dx = (vx[sb] - vx[sa]) * inv_n;
          dvy_dx = (vy[sb] - vy[sa]) * inv_n;
          dvx_dy = ((vx[sb + PW] + vx[sa + PW]) - (vx[sb - PW] + vx[sa - PW])) * inv_t;
          dvy_dy = ((vy[sb + PW] + vy[sa + PW]) - (vy[sb - PW] + vy[sa - PW])) * inv_t;
        } else {
          const R inv_n = static_cast<R>(p.inv_dy), inv_t = static_cast<R>(p.inv_4dx);
          dvx_dy = (vx[sb] - vx[sa]) * inv_n;
          dvy_dy = (vy[sb] - vy[sa]) * inv_n;
          dvx_dx = ((vx[sb + 1] + vx[sa + 1]) - (vx[sb - 1] + vx[sa - 1])) * inv_t;
          dvy_dx = ((vy[sb + 1] + vy[sa + 1]) - (vy[sb - 1] + vy[sa - 1])) * inv_t;
        }
        const R shear = dvy_dx + dvx_dy;
        R s0, s1;
        if (xs) {
          s0 = R(4.0 / 3.0) * dvx_dx - R(2.0 / 3.0) * dvy_dy;
          s1 = shear;
        } else {
          s0 = shear;
          s1 = R(4.0 / 3.0) * dvy_dy - R(2.0 / 3.0) * dvx_dx;
        }
        R nu = static_cast<R>(p.nu);
        if (p.smag_on) {
          const R s2 = R(2) * (dvx_dx * dvx_dx + dvy_dy * dvy_dy) + shear * shear;
          nu = nu + static_cast<R>(p.smag_c) * sqrt(s2);
        }
        const R mu = (R(0.5) * nu) * (sW[sb] + sW[sa]);
        f1 = f1 + -(mu * s0);
        f2 = f2 + -(mu * s1);
      }
      if (tau != nullptr) {
        const int gy = wrap_index(y0 + r, p.ny), gx = wrap_index(x0 + c, p.nx);
        const int ay = xs ? gy : wrap_index(y0 + r - 1, p.ny);
        const int ax = xs ? wrap_index(x0 + c - 1, p.nx) : gx;
        const R* tb = tau + ((size_t)gy * p.nx + gx) * 3;
        const R* ta = tau + ((size_t)ay * p.nx + ax) * 3;
        const int k0 = xs ? 0 : 1;
        f1 = f1 + R(0.5) * (ta[k0] + tb[k0]);
        f2 = f2 + R(0.5) * (ta[k0 + 1] + tb[k0 + 1]);
      }

      const bool own = xs ? c < tw : r < th;  // the face is the low face of a tile cell
      if (p.trace_on && own) {
        const size_t cell = ((size_t)(y0 + r) * p.nx + (x0 + c)) * NV;
        R* tl_out = static_cast<R*>(xs ? p.trace.left_x : p.trace.left_y);
        R* tr_out = static_cast<R*>(xs ? p.trace.right_x : p.trace.right_y);
        for (int v = 0; v < NV; ++v) {
          if (tl_out) tl_out[cell + v] = L[v * fplane + fo];
          if (tr_out) tr_out[cell + v] = Rt[v * fplane + fo];
        }
      }
      L[fo] = f0;
      L[fplane + fo] = f1;
      L[2 * fplane + fo] = f2;
      for (int v = 3; v < NV; ++v) {
        const R up = f0 >= R(0) ? L[v * fplane + fo] : Rt[v * fplane + fo];
        L[v * fplane + fo] = f0 * up;
      }
      if (p.trace_on && own) {
        R* tf = static_cast<R*>(xs ? p.trace.flux_x : p.trace.flux_y);
        if (tf) {
          const size_t cell = ((size_t)(y0 + r) * p.nx + (x0 + c)) * NV;
          for (int v = 0; v < NV; ++v) tf[cell + v] = L[v * fplane + fo];
        }
      }
    }
  }
  __syncthreads();

  // ---- phase 3: divergence, RK combine, drag, floor, write-back -----------
  const R* __restrict__ V = static_cast<const R*>(p.V);
  R* Uo = static_cast<R*>(p.Uout);
  R* Vo = static_cast<R*>(p.Vout);
  const double dt = p.clock->dt;
  const R sdt = static_cast<R>(p.beta * dt);
  const R g0 = static_cast<R>(p.g0), g1 = static_cast<R>(p.g1), delta = static_cast<R>(p.delta);
  const R inv_dx = static_cast<R>(p.inv_dx), inv_dy = static_cast<R>(p.inv_dy);
  const R kdrag = sdt * static_cast<R>(p.drag);
  const R cs = static_cast<R>(p.cs);
  double vmax[2] = {0.0, 0.0};
  for (int idx = tid; idx < th * tw; idx += kStageThreads) {
    const int r = idx / tw, c = idx - r * tw;
    const size_t cell = ((size_t)(y0 + r) * p.nx + (x0 + c)) * NV;
    const int sw = (r + H) * PW + (c + H);
    const R rho_in = sW[sw];
    R out0 = R(0), out1 = R(0), out2 = R(0);
    for (int v = 0; v < NV; ++v) {
      const int fx = v * fxplane + r * fxp + c;
      const int fy = v * fyplane + r * TX + c;
      const R div = (sLx[fx + 1] - sLx[fx]) * inv_dx + (sLy[fy + TX] - sLy[fy]) * inv_dy;
      const R u = v == 0 ? rho_in : U[cell + v];
      R vs = V[cell + v];
      if (v == 0 && p.floor_v) vs = vs < dfloor ? dfloor : vs;
      if (p.has_delta) {
        vs = vs + delta * u;
        if (Vo) Vo[cell + v] = vs;
      }
      R un = p.blend ? vs + (g0 * (u - vs) - sdt * div) : g0 * u + g1 * vs - sdt * div;
      if (p.drag_on && (v == 1 || v == 2)) un = un + -((kdrag * rho_in) * sW[v * wplane + sw]);
      if (p.trace_on) {
        if (p.trace.saved) static_cast<R*>(p.trace.saved)[cell + v] = vs;
        if (p.trace.conserved) static_cast<R*>(p.trace.conserved)[cell + v] = un;
        if (p.trace.primitives) static_cast<R*>(p.trace.primitives)[cell + v] = sW[v * wplane + sw];
      }
      if (v == 0) {
        if (p.floor_out) un = un < dfloor ? dfloor : un;
        out0 = un;
      } else if (v == 1) {
        out1 = un;
      } else if (v == 2) {
        out2 = un;
      }
      Uo[cell + v] = un;
    }
    if (p.want_cfl) {
      const R inv = R(1) / out0;
      vmax[0] = nan_max(vmax[0], static_cast<double>(fabs(inv * out1) + cs));
      vmax[1] = nan_max(vmax[1], static_cast<double>(fabs(inv * out2) + cs));
    }
  }
  if (p.want_cfl) {
    block_nan_max<2>(vmax, red);
    if (tid == 0) {
      p.partials[(size_t)blockIdx.x * kCflSlots + 0] = vmax[0];
      p.partials[(size_t)blockIdx.x * kCflSlots + 1] = vmax[1];
      p.partials[(size_t)blockIdx.x * kCflSlots + 2] = 0.0;
      if (blockIdx.x == 0) p.header->n_cfl = gridDim.x;
    }
  }
}

template <typename R, int RECON, int RS>
cudaError_t launch_stage_one(const StageParams& p, dim3 grid, size_t smem, cudaStream_t s) {
  auto kernel = stage_kernel<R, RECON, RS>;
  // The opt-in shared-memory limit is a per-device function attribute; raise
  // it once per device to the largest tile requested so far.
  static int granted[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if ((int)smem > granted[dev]) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    granted[dev] = (int)smem;
  }
  kernel<<<grid, kStageThreads, smem, s>>>(p);
  return cudaGetLastError();
}

// Standalone face states (fluxes.py:126-131 reconstruct_faces) for one axis:
// left/right at the low face of every cell, recomputing both neighbours'
// edges per face. Used by the operator-level API, not by the fused step.
template <typename R, int RECON>
__global__ void face_states_kernel(const R* __restrict__ W, int ny, int nx, int nv, int axis, R dfloor,
                                   R* __restrict__ left, R* __restrict__ right) {
  const int64_t n = (int64_t)ny * nx * nv;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int v = (int)(k % nv);
  const int64_t cell = k / nv;
  const int j = (int)(cell / nx), i = (int)(cell - (int64_t)j * nx);
  auto at = [&](int o) -> R {  // W at offset o along the axis
    const int jj = axis == 0 ? wrap_index(j + o, ny) : j;
    const int ii = axis == 1 ? wrap_index(i + o, nx) : i;
    return W[((int64_t)jj * nx + ii) * nv + v];
  };
  R lo, hi, lo_prev, hi_prev;
  edges<RECON>(at(-2), at(-1), at(0), at(1), at(2), lo, hi);
  edges<RECON>(at(-3), at(-2), at(-1), at(0), at(1), lo_prev, hi_prev);
  if ((RECON == JX_PPMX || RECON == JX_WENOZ) && v == 0) {
    hi_prev = fmax(hi_prev, dfloor);
    lo = fmax(lo, dfloor);
  }
  left[k] = hi_prev;
  right[k] = lo;
}

template <int RECON>
cudaError_t launch_face_states_recon(int dtype, const void* W, int ny, int nx, int nv, int axis,
                                     double dfloor, void* left, void* right, cudaStream_t s) {
  const int64_t n = (int64_t)ny * nx * nv;
  if (n == 0) return cudaSuccess;
  const int g = (int)((n + 255) / 256);
  if (dtype == JX_F64)
    face_states_kernel<double, RECON><<<g, 256, 0, s>>>((const double*)W, ny, nx, nv, axis, dfloor,
                                                        (double*)left, (double*)right);
  else
    face_states_kernel<float, RECON><<<g, 256, 0, s>>>((const float*)W, ny, nx, nv, axis, (float)dfloor,
                                                       (float*)left, (float*)right);
  return cudaGetLastError();
}

template <int RECON>
cudaError_t launch_stage_recon(int dtype, int rsolver, const StageParams& p, dim3 grid, size_t smem,
                               cudaStream_t s) {
  if (dtype == JX_F64) {
    switch (rsolver) {
      case JX_LLF: return launch_stage_one<double, RECON, JX_LLF>(p, grid, smem, s);
      case JX_HLLE: return launch_stage_one<double, RECON, JX_HLLE>(p, grid, smem, s);
      case JX_ROE: return launch_stage_one<double, RECON, JX_ROE>(p, grid, smem, s);
    }
  } else {
    switch (rsolver) {
      case JX_LLF: return launch_stage_one<float, RECON, JX_LLF>(p, grid, smem, s);
      case JX_HLLE: return launch_stage_one<float, RECON, JX_HLLE>(p, grid, smem, s);
      case JX_ROE: return launch_stage_one<float, RECON, JX_ROE>(p, grid, smem, s);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace jx
