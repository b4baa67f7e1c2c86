// The fused RK-stage kernel: one CTA owns a TX x TY tile of cells.
//
//   load    the tile plus a periodic ghost halo of depth H from U, floor rho
//           and convert to primitives W in shared memory
//           (recover_isothermal, hydro.py:54-60);
//   then, for the x sweep and then the y sweep:
//     faces   PPM4/PPMX only: the limited value at every face the tile needs,
//             computed once and shared by the two cells that meet there
//             (fluxes.py:29-32, 62-68);
//     edges   each cell's low/high edge values (fluxes.py:6-131), written
//             as the right state of its low face and the left state of its
//             high face;
//     solve   the Riemann flux of every face (fluxes.py:134-219) plus the
//             viscous/Smagorinsky stress (fluxes.py:227-266) and the SGS
//             stress (fluxes.py:269-280), kept in shared memory;
//   update  flux divergence (fluxes.py:283-287), RK combine (hydro.py:39-51),
//           drag (hydro.py:122-125), density floor (hydro.py:143), write-back,
//           and on the last stage the CFL partial max of the new state.
//
// Only the stage output (and the RK4 saved register) goes back to HBM.
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"

namespace jx {

// Shared-memory views of one tile (all planes variable-major).
template <typename R> struct Tile {
  R *W, *Fx, *Fy, *A, *Rt;
  int wplane, fxplane, fyplane, aplane, rplane;
  int PW, TX;
};

// Index helpers for a sweep along DIR (0 = x, 1 = y). A "line" is a tile row
// (x sweep) or column (y sweep); q is the position along it.
template <int DIR> struct Sweep {
  // face q of line ln in the flux/right-state planes
  static __device__ __forceinline__ int face(int ln, int q, int TX) { return DIR == 0 ? ln * (TX + 1) + q : q * TX + ln; }
  // face q (q >= -1) of line ln in the face-value plane
  static __device__ __forceinline__ int aface(int ln, int q, int TX) { return DIR == 0 ? ln * (TX + 3) + q + 1 : (q + 1) * TX + ln; }
  // cell q of line ln in the primitive plane (q may be negative)
  static __device__ __forceinline__ int cell(int ln, int q, int PW, int H) {
    return DIR == 0 ? (ln + H) * PW + (q + H) : (q + H) * PW + (ln + H);
  }
  static __device__ __forceinline__ int stride(int PW) { return DIR == 0 ? 1 : PW; }
};

template <typename R, int RECON, int RS, int DIR>
__device__ __forceinline__ void sweep(const StageParams& p, const StageConsts<R>& k, Tile<R>& t, int x0, int y0,
                                      int tw, int th) {
  using S = Sweep<DIR>;
  using Tr = ReconTraits<RECON>;
  constexpr int H = Tr::kHalo;
  constexpr bool kFaceFloor = RECON == 3 || RECON == 4;  // fluxes.py:128-130
  const int tid = threadIdx.x;
  const int NV = p.nv, PW = t.PW, TX = t.TX;
  const int nline = DIR == 0 ? th : tw;  // lines in this sweep
  const int n = DIR == 0 ? tw : th;      // cells per line
  const int st = S::stride(PW);
  R* F = DIR == 0 ? t.Fx : t.Fy;
  const int fplane = DIR == 0 ? t.fxplane : t.fyplane;
  // Thread -> (line, position): consecutive threads walk along x.
  auto split = [&](int idx, int len, int& ln, int& q) {
    if (DIR == 0) { ln = idx / len; q = idx - ln * len; }
    else { ln = idx % nline; q = idx / nline; }
  };

  // ---- face values shared by neighbouring cells (PPM4 / PPMX) ------------
  if constexpr (Tr::kFaceShared) {
    const int len = n + 3;  // faces -1 .. n+1
    for (int idx = tid; idx < nline * len; idx += kStageThreads) {
      int ln, q;
      split(idx, len, ln, q);
      q -= 1;
      const int s = S::cell(ln, q, PW, H);  // cell on the high side of face q
      for (int v = 0; v < NV; ++v) {
        const R* w = t.W + v * t.wplane + s;
        t.A[v * t.aplane + S::aface(ln, q, TX)] = face_value<RECON>(w[-2 * st], w[-st], w[0], w[st]);
      }
    }
    __syncthreads();
  }

  // ---- cell edges -> right state of the low face, left state of the high face
  {
    const int len = n + 2;  // cells -1 .. n
    for (int idx = tid; idx < nline * len; idx += kStageThreads) {
      int ln, q;
      split(idx, len, ln, q);
      q -= 1;
      const int s = S::cell(ln, q, PW, H);
      for (int v = 0; v < NV; ++v) {
        const R* w = t.W + v * t.wplane + s;
        const R c = w[0];
        const R m1 = H >= 2 ? w[-st] : c;
        const R p1 = H >= 2 ? w[st] : c;
        const R m2 = H >= 3 ? w[-2 * st] : c;
        const R p2 = H >= 3 ? w[2 * st] : c;
        R lf = R(0), hf = R(0);
        if constexpr (Tr::kFaceShared) {
          lf = t.A[v * t.aplane + S::aface(ln, q, TX)];
          hf = t.A[v * t.aplane + S::aface(ln, q + 1, TX)];
        }
        R lo, hi;
        cell_edges<RECON>(m2, m1, c, p1, p2, lf, hf, lo, hi);
        if (kFaceFloor && v == 0) {
          lo = Num<R>::max(lo, k.dfloor);
          hi = Num<R>::max(hi, k.dfloor);
        }
        if (q + 1 <= n) F[v * fplane + S::face(ln, q + 1, TX)] = hi;   // left state of face q+1
        if (q >= 0) t.Rt[v * t.rplane + S::face(ln, q, TX)] = lo;      // right state of face q
      }
    }
    __syncthreads();
  }

  // ---- Riemann solve + viscous + SGS stress --------------------------------
  {
    Gas<R> gas;
    gas.cs = k.cs;
    gas.cs2 = k.cs2;
    gas.inv_cs = k.inv_cs;
    gas.half_inv_cs = k.half_inv_cs;
    gas.quarter_inv_cs = R(0.5) * k.half_inv_cs;
    const R* __restrict__ tau = static_cast<const R*>(p.tau);
    const int len = n + 1;  // faces 0 .. n
    constexpr int nn = DIR == 0 ? 1 : 2, tt = DIR == 0 ? 2 : 1;
    for (int idx = tid; idx < nline * len; idx += kStageThreads) {
      int ln, q;
      split(idx, len, ln, q);
      const int fo = S::face(ln, q, TX);
      R* L = F + fo;
      R* Rr = t.Rt + fo;
      R f0, fn, ft;
      riemann<RS>(L[0], Rr[0], L[nn * fplane], Rr[nn * t.rplane], L[tt * fplane], Rr[tt * t.rplane], gas, f0, fn,
                  ft);
      R f1 = DIR == 0 ? fn : ft;
      R f2 = DIR == 0 ? ft : fn;
      const int r = DIR == 0 ? ln : q, c = DIR == 0 ? q : ln;  // tile row/column of the face's cell

      if (p.visc_on) {
        // Cell b on the high side of the face, a on the low side.
        const int sb = (r + H) * PW + (c + H);
        const int sa = sb - S::stride(PW);
        const R* vx = t.W + t.wplane;
        const R* vy = t.W + 2 * t.wplane;
        const int ts = DIR == 0 ? PW : 1;  // transverse neighbours
        viscous_face<DIR, R>(p.smag_on, k.nu, k.smag_c, DIR == 0 ? k.inv_dx : k.inv_dy,
                             DIR == 0 ? k.inv_4dy : k.inv_4dx, t.W[sa], t.W[sb], vx[sa], vy[sa], vx[sb], vy[sb],
                             vx[sb + ts] + vx[sa + ts], vy[sb + ts] + vy[sa + ts], vx[sb - ts] + vx[sa - ts],
                             vy[sb - ts] + vy[sa - ts], f1, f2);
      }
      if (tau != nullptr) {
        const int gy = wrap_index(y0 + r, p.ny), gx = wrap_index(x0 + c, p.nx);
        const int ay = DIR == 0 ? gy : wrap_index(y0 + r - 1, p.ny);
        const int ax = DIR == 0 ? wrap_index(x0 + c - 1, p.nx) : gx;
        const R* tb = tau + ((size_t)gy * p.nx + gx) * 3;
        const R* ta = tau + ((size_t)ay * p.nx + ax) * 3;
        constexpr int k0 = DIR == 0 ? 0 : 1;
        f1 = add_half_sum(f1, ta[k0], tb[k0]);
        f2 = add_half_sum(f2, ta[k0 + 1], tb[k0 + 1]);
      }

      const bool own = q < n;  // the low face of a cell of this tile
      if (p.trace_on && own) {
        const size_t cell = ((size_t)(y0 + r) * p.nx + (x0 + c)) * NV;
        R* tl_out = static_cast<R*>(DIR == 0 ? p.trace.left_x : p.trace.left_y);
        R* tr_out = static_cast<R*>(DIR == 0 ? p.trace.right_x : p.trace.right_y);
        for (int v = 0; v < NV; ++v) {
          if (tl_out) tl_out[cell + v] = L[v * fplane];
          if (tr_out) tr_out[cell + v] = Rr[v * t.rplane];
        }
      }
      L[0] = f0;
      L[fplane] = f1;
      L[2 * fplane] = f2;
      for (int v = 3; v < NV; ++v) {
        const R up = Num<R>::ge0(f0) ? L[v * fplane] : Rr[v * t.rplane];
        L[v * fplane] = Ops<R>::mul(f0, up);
      }
      if (p.trace_on && own) {
        R* tf = static_cast<R*>(DIR == 0 ? p.trace.flux_x : p.trace.flux_y);
        if (tf) {
          const size_t cell = ((size_t)(y0 + r) * p.nx + (x0 + c)) * NV;
          for (int v = 0; v < NV; ++v) tf[cell + v] = L[v * fplane];
        }
      }
    }
    __syncthreads();
  }
}

template <typename R, int RECON, int RS>
__global__ void __launch_bounds__(kStageThreads) stage_kernel(const StageParams p) {
  if (p.clock->done) return;
  using N = Num<R>;
  constexpr int H = ReconTraits<RECON>::kHalo;
  const StageConsts<R>& k = stage_consts<R>(p);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32 * 2];
  __shared__ R s_sdt;

  const int tid = threadIdx.x;
  const int NV = p.nv, TX = p.tx, TY = p.ty;
  const int bx = blockIdx.x % p.tiles_x, by = blockIdx.x / p.tiles_x;
  const int x0 = bx * TX, y0 = by * TY;
  const int tw = min(TX, p.nx - x0), th = min(TY, p.ny - y0);
  const TilePlanes pl = tile_planes(RECON, TX, TY);
  Tile<R> t;
  t.PW = pl.pw;
  t.TX = TX;
  t.wplane = pl.w;
  t.fxplane = pl.fx;
  t.fyplane = pl.fy;
  t.aplane = pl.a;
  t.rplane = pl.r;
  t.W = reinterpret_cast<R*>(smem_raw);
  t.Fx = t.W + NV * pl.w;
  t.Fy = t.Fx + NV * pl.fx;
  t.A = t.Fy + NV * pl.fy;
  t.Rt = t.A + NV * pl.a;
  const int PW = pl.pw;

  const R* __restrict__ U = static_cast<const R*>(p.U);
  if (tid == 0) s_sdt = static_cast<R>(p.beta * p.clock->dt);

  // ---- load + primitive recovery -----------------------------------------
  const int lw = tw + 2 * H, lh = th + 2 * H;
  for (int idx = tid; idx < lw * lh; idx += kStageThreads) {
    const int ly = idx / lw, lx = idx - ly * lw;
    const int gy = wrap_index(y0 + ly - H, p.ny), gx = wrap_index(x0 + lx - H, p.nx);
    const R* u = U + ((size_t)gy * p.nx + gx) * NV;
    R rho = u[0];
    rho = N::lt(rho, k.dfloor) ? k.dfloor : rho;
    const R inv = Num<R>::rcp(rho);
    const int s = ly * PW + lx;
    t.W[s] = rho;
    for (int v = 1; v < NV; ++v) t.W[v * t.wplane + s] = Ops<R>::mul(inv, u[v]);
  }
  __syncthreads();

  sweep<R, RECON, RS, 0>(p, k, t, x0, y0, tw, th);
  sweep<R, RECON, RS, 1>(p, k, t, x0, y0, tw, th);

  // ---- divergence, RK combine, drag, floor, write-back -------------------
  const R* __restrict__ V = static_cast<const R*>(p.V);
  R* Uo = static_cast<R*>(p.Uout);
  R* Vo = static_cast<R*>(p.Vout);
  const R sdt = s_sdt;
  const R kdrag = sdt * k.drag;
  const R ncx = -(sdt * k.inv_dx), ncy = -(sdt * k.inv_dy);
  R vmax0 = R(0), vmax1 = R(0);
  for (int idx = tid; idx < th * tw; idx += kStageThreads) {
    const int r = idx / tw, c = idx - r * tw;
    const size_t cell = ((size_t)(y0 + r) * p.nx + (x0 + c)) * NV;
    const int sw = (r + H) * PW + (c + H);
    const R rho_in = t.W[sw];
    R out0 = R(0), out1 = R(0), out2 = R(0);
    for (int v = 0; v < NV; ++v) {
      const int fx = v * t.fxplane + r * (TX + 1) + c;
      const int fy = v * t.fyplane + r * TX + c;
      const R u = v == 0 ? rho_in : U[cell + v];
      R vs = V[cell + v];
      if (v == 0 && p.floor_v) vs = N::lt(vs, k.dfloor) ? k.dfloor : vs;
      if (p.has_delta) {
        vs = delta_update(vs, k.delta, u);
        if (Vo) Vo[cell + v] = vs;
      }
      R un = rk_combine<R>(p.blend, k.g0, k.g1, u, vs, t.Fx[fx + 1] - t.Fx[fx], t.Fy[fy + TX] - t.Fy[fy], ncx, ncy);
      if (p.drag_on && (v == 1 || v == 2)) un = drag_term(un, kdrag * rho_in, t.W[v * t.wplane + sw]);
      if (p.trace_on) {
        if (p.trace.saved) static_cast<R*>(p.trace.saved)[cell + v] = vs;
        if (p.trace.conserved) static_cast<R*>(p.trace.conserved)[cell + v] = un;
        if (p.trace.primitives) static_cast<R*>(p.trace.primitives)[cell + v] = t.W[v * t.wplane + sw];
      }
      if (v == 0) {
        if (p.floor_out) un = N::lt(un, k.dfloor) ? k.dfloor : un;
        out0 = un;
      } else if (v == 1) {
        out1 = un;
      } else if (v == 2) {
        out2 = un;
      }
      Uo[cell + v] = un;
    }
    if (p.want_cfl) {
      // Both candidates are >= cs > 0 or NaN: an ordered max that keeps NaN.
      const R inv = Num<R>::rcp(out0);
      vmax0 = N::nanmax_pos(vmax0, signal_speed(inv, out1, k.cs));
      vmax1 = N::nanmax_pos(vmax1, signal_speed(inv, out2, k.cs));
    }
  }
  if (p.want_cfl) {
    double vmax[2] = {static_cast<double>(vmax0), static_cast<double>(vmax1)};
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
  const int64_t kk = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= n) return;
  const int v = (int)(kk % nv);
  const int64_t cell = kk / nv;
  const int j = (int)(cell / nx), i = (int)(cell - (int64_t)j * nx);
  auto at = [&](int o) -> R {  // W at offset o along the axis
    const int jj = axis == 0 ? wrap_index(j + o, ny) : j;
    const int ii = axis == 1 ? wrap_index(i + o, nx) : i;
    return W[((int64_t)jj * nx + ii) * nv + v];
  };
  R lo, hi, lo_prev, hi_prev;
  edges_from_stencil<RECON>(at(-3), at(-2), at(-1), at(0), at(1), at(2), at(3), lo, hi);
  edges_from_stencil<RECON>(at(-4), at(-3), at(-2), at(-1), at(0), at(1), at(2), lo_prev, hi_prev);
  if ((RECON == JX_PPMX || RECON == JX_WENOZ) && v == 0 && dfloor == dfloor) {
    hi_prev = Num<R>::max(hi_prev, dfloor);
    lo = Num<R>::max(lo, dfloor);
  }
  left[kk] = hi_prev;
  right[kk] = lo;
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
