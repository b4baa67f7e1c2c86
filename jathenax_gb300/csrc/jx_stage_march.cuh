// Register-marching variant of the fused RK-stage kernel (3 or 4 variables),
// built for float32, where the shared-memory tile kernel is bound by
// instruction issue rather than by arithmetic or HBM.
//
// One warp updates one tile of kMarchTileX (58) columns by StageParams::ty
// rows. Lane l holds the two adjacent columns 2l and 2l+1 of a 64-column
// strip (3 ghost columns on each side) and walks down the rows, keeping a
// 5-row window of primitives in registers:
//   * the y sweep runs along the walk: as row j arrives, the shared face
//     value between rows j-2 and j-1, the edges of row j-2 and the Riemann
//     flux of the face below row j-2 are computed, carrying the previous face
//     value, upper edge and flux in registers;
//   * the x sweep of row j-3 runs across the lanes: each lane evaluates two
//     face values, both cells' edges and two Riemann problems; neighbour
//     values cross lanes by warp shuffles (four cells, one face value, one
//     edge and one flux per row);
//   * row j-3 is then updated (divergence, RK combine, drag, floor) and
//     written for the tile's 58 columns.
// There is no shared memory and no barrier; a warp's CFL partial (the exact
// maximum over its tile) goes to the workspace slot of its tile. Arithmetic
// per cell is the same as in jx_stage_fast.cuh (same device functions in the
// same order), so results agree with it to rounding.
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"
#include "jx_stage_fast.cuh"

namespace jx {

template <typename R, int NV>
__device__ __forceinline__ Cell4<R> shfl_up_cell(const Cell4<R>& c, int d) {
  Cell4<R> o;
#pragma unroll
  for (int v = 0; v < 4; ++v) o.v[v] = v < NV ? __shfl_up_sync(0xffffffffu, c.v[v], d) : R(0);
  return o;
}

template <typename R, int NV>
__device__ __forceinline__ Cell4<R> shfl_down_cell(const Cell4<R>& c, int d) {
  Cell4<R> o;
#pragma unroll
  for (int v = 0; v < 4; ++v) o.v[v] = v < NV ? __shfl_down_sync(0xffffffffu, c.v[v], d) : R(0);
  return o;
}

template <typename R, int NV>
__device__ __forceinline__ Cell4<R> recover_cell(const Cell4<R>& u, R dfloor) {
  Cell4<R> w;
  const R rho = Num<R>::lt(u.v[0], dfloor) ? dfloor : u.v[0];
  const R inv = Num<R>::rcp(rho);
  w.v[0] = rho;
#pragma unroll
  for (int v = 1; v < 4; ++v) w.v[v] = v < NV ? inv * u.v[v] : R(0);
  return w;
}

template <int RECON, typename R, int NV>
__device__ __forceinline__ void edges_cells(const Cell4<R>& m2, const Cell4<R>& m1, const Cell4<R>& c,
                                            const Cell4<R>& p1, const Cell4<R>& p2, const Cell4<R>& lf,
                                            const Cell4<R>& hf, R dfloor, Cell4<R>& lo, Cell4<R>& hi) {
#pragma unroll
  for (int v = 0; v < NV; ++v)
    cell_edges<RECON>(m2.v[v], m1.v[v], c.v[v], p1.v[v], p2.v[v], lf.v[v], hf.v[v], lo.v[v], hi.v[v]);
#pragma unroll
  for (int v = NV; v < 4; ++v) lo.v[v] = hi.v[v] = R(0);
  if constexpr (RECON == 3 || RECON == 4) {  // fluxes.py:128-130
    lo.v[0] = Num<R>::max(lo.v[0], dfloor);
    hi.v[0] = Num<R>::max(hi.v[0], dfloor);
  }
}

template <int RECON, typename R, int NV>
__device__ __forceinline__ Cell4<R> faces_cells(const Cell4<R>& w0, const Cell4<R>& w1, const Cell4<R>& w2,
                                                const Cell4<R>& w3) {
  Cell4<R> a;
#pragma unroll
  for (int v = 0; v < NV; ++v) a.v[v] = face_value<RECON>(w0.v[v], w1.v[v], w2.v[v], w3.v[v]);
#pragma unroll
  for (int v = NV; v < 4; ++v) a.v[v] = R(0);
  return a;
}

// Riemann flux (x/y component order) plus passive-scalar upwinding.
template <int RS, int DIR, typename R, int NV>
__device__ __forceinline__ Cell4<R> face_flux_cells(const Cell4<R>& L, const Cell4<R>& Rv, const Gas<R>& gas) {
  constexpr int nn = DIR == 0 ? 1 : 2, tt = DIR == 0 ? 2 : 1;
  R f0, fn, ft;
  riemann<RS>(L.v[0], Rv.v[0], L.v[nn], Rv.v[nn], L.v[tt], Rv.v[tt], gas, f0, fn, ft);
  Cell4<R> f;
  f.v[0] = f0;
  f.v[1] = DIR == 0 ? fn : ft;
  f.v[2] = DIR == 0 ? ft : fn;
  f.v[3] = R(0);
#pragma unroll
  for (int v = 3; v < NV; ++v) f.v[v] = f0 * (Num<R>::ge0(f0) ? L.v[v] : Rv.v[v]);
  return f;
}

// Viscous momentum flux at a face (fluxes.py:227-266) from the velocities of
// the two cells a (low side) and b (high side) and the transverse difference
// ((b+ + a+) - (b- + a-)); rho_a, rho_b their densities.
template <int DIR, typename R>
__device__ __forceinline__ void viscous_add(const StageParams& p, const StageConsts<R>& k, R rho_a, R rho_b,
                                            R ax, R ay, R bx, R by, R tpx, R tpy, R tmx, R tmy, Cell4<R>& f) {
  R dvx_dx, dvy_dx, dvx_dy, dvy_dy;
  if (DIR == 0) {
    dvx_dx = (bx - ax) * k.inv_dx;
    dvy_dx = (by - ay) * k.inv_dx;
    dvx_dy = (tpx - tmx) * k.inv_4dy;
    dvy_dy = (tpy - tmy) * k.inv_4dy;
  } else {
    dvx_dy = (bx - ax) * k.inv_dy;
    dvy_dy = (by - ay) * k.inv_dy;
    dvx_dx = (tpx - tmx) * k.inv_4dx;
    dvy_dx = (tpy - tmy) * k.inv_4dx;
  }
  const R shear = dvy_dx + dvx_dy;
  R s0, s1;
  if (DIR == 0) {
    s0 = R(4.0 / 3.0) * dvx_dx - R(2.0 / 3.0) * dvy_dy;
    s1 = shear;
  } else {
    s0 = shear;
    s1 = R(4.0 / 3.0) * dvy_dy - R(2.0 / 3.0) * dvx_dx;
  }
  R nu = k.nu;
  if (p.smag_on) {
    const R s2 = R(2) * (dvx_dx * dvx_dx + dvy_dy * dvy_dy) + shear * shear;
    nu = nu + k.smag_c * sqrt(s2);
  }
  const R mu = (R(0.5) * nu) * (rho_b + rho_a);
  f.v[1] = f.v[1] + -(mu * s0);
  f.v[2] = f.v[2] + -(mu * s1);
}

// Both columns of one lane: a 5-row window of primitives (rows j-4 .. j),
// the face value below row j-1, the upper edge of row j-3 and the y flux
// below row j-3 (see the file comment).
template <typename R> struct MarchColumn {
  Cell4<R> W4, W3, W2, W1, W0, Ay2, hy3, Fy3;
};

// PREFETCH_V: issue L2 prefetches of the saved register two rows ahead of
// the RK combine. Measured on GB300: it helps the batch kernel (12 resident
// warps per SM, ensemble cycle -2.2 %) and costs the single-solve kernel
// (16 warps, already hiding the latency; +2.4 % at 4096²). Results do not
// depend on it.
template <typename R, int RECON, int RS, int NV, bool PREFETCH_V>
__device__ __forceinline__ void march_tile(const StageParams& p, int tile, int ntiles) {
  using N = Num<R>;
  const StageConsts<R>& k = stage_consts<R>(p);
  const int lane = threadIdx.x & 31;
  const int TY = p.ty;
  const int bx = tile % p.tiles_x, by = tile / p.tiles_x;
  const int x0 = bx * kMarchTileX;  // first output column of the tile
  const int y0 = by * TY;
  const int c0 = x0 - 3 + 2 * lane;  // this lane's columns: c0 and c0 + 1
  const int gx[2] = {wrap_fast(c0, p.nx), wrap_fast(c0 + 1, p.nx)};
  // Local columns 3 .. 3 + kMarchTileX - 1 of the 64 are written.
  const bool out[2] = {lane >= 2 && lane <= 30 && c0 < p.nx, lane >= 1 && lane <= 29 && c0 + 1 < p.nx};
  const R* __restrict__ U = static_cast<const R*>(p.U);
  const R* __restrict__ V = static_cast<const R*>(p.V);
  R* Uo = static_cast<R*>(p.Uout);
  R* Vo = static_cast<R*>(p.Vout);
  const R* __restrict__ tau = static_cast<const R*>(p.tau);
  Gas<R> gas;
  gas.cs = k.cs;
  gas.cs2 = k.cs2;
  gas.inv_cs = k.inv_cs;
  gas.half_inv_cs = k.half_inv_cs;
  gas.quarter_inv_cs = R(0.5) * k.half_inv_cs;
  const R sdt = static_cast<R>(p.beta * p.clock->dt);
  const R kdrag = sdt * k.drag;
  const R ncx = -(sdt * k.inv_dx), ncy = -(sdt * k.inv_dy);
  constexpr unsigned kAll = 0xffffffffu;

  MarchColumn<R> col[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) col[h].W4 = col[h].W3 = col[h].W2 = col[h].W1 = col[h].W0 = col[h].Ay2 =
      col[h].hy3 = col[h].Fy3 = Cell4<R>{};
  R vmax0 = R(0), vmax1 = R(0);
  const int iters = TY + 6;
  Cell4<R> next[2];
  {
    const size_t row = (size_t)wrap_fast(y0 - 3, p.ny) * p.nx;
#pragma unroll
    for (int h = 0; h < 2; ++h) next[h] = load_cell<R, NV>(U + (row + gx[h]) * NV);
  }
  for (int it = 0; it < iters; ++it) {
    const int j = y0 - 3 + it;
    // ---- y sweep of both columns -------------------------------------------
    Cell4<R> Ay1[2], lo[2], hi[2], Fy2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      MarchColumn<R>& c = col[h];
      c.W4 = c.W3;
      c.W3 = c.W2;
      c.W2 = c.W1;
      c.W1 = c.W0;
      c.W0 = recover_cell<R, NV>(next[h], k.dfloor);
    }
    if (it + 1 < iters) {
      const size_t row = (size_t)wrap_fast(j + 1, p.ny) * p.nx;
#pragma unroll
      for (int h = 0; h < 2; ++h) next[h] = load_cell<R, NV>(U + (row + gx[h]) * NV);
    }
    // The saved register V is read once, by the RK combine of row j-3; ask L2
    // for row j-1 now (two rows ahead, no registers held) so that the combine
    // does not wait for DRAM. Only cells the combine will read.
    if (PREFETCH_V && it >= 4 && j - 1 < p.ny && j - 1 < y0 + TY) {
      const size_t row = (size_t)(j - 1) * p.nx;
#pragma unroll
      for (int h = 0; h < 2; ++h)
        if (out[h]) asm volatile("prefetch.global.L2 [%0];" ::"l"(V + (row + (size_t)(c0 + h)) * NV));
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      MarchColumn<R>& c = col[h];
      Ay1[h] = c.Ay2;
      if (it >= 3 && ReconTraits<RECON>::kFaceShared) Ay1[h] = faces_cells<RECON, R, NV>(c.W3, c.W2, c.W1, c.W0);
      hi[h] = c.hy3;
      lo[h] = c.hy3;
      if (it >= 4) edges_cells<RECON, R, NV>(c.W4, c.W3, c.W2, c.W1, c.W0, c.Ay2, Ay1[h], k.dfloor, lo[h], hi[h]);
      Fy2[h] = c.Fy3;
    }
    if (it >= 5) {
      // Faces between rows j-3 (a) and j-2 (b).
#pragma unroll
      for (int h = 0; h < 2; ++h) Fy2[h] = face_flux_cells<RS, 1, R, NV>(col[h].hy3, lo[h], gas);
      if (p.visc_on) {
        // Transverse x differences: columns c-1 and c+1 of rows j-3 and j-2.
        const R lbx = __shfl_up_sync(kAll, col[1].W2.v[1], 1), lax = __shfl_up_sync(kAll, col[1].W3.v[1], 1);
        const R lby = __shfl_up_sync(kAll, col[1].W2.v[2], 1), lay = __shfl_up_sync(kAll, col[1].W3.v[2], 1);
        const R rbx = __shfl_down_sync(kAll, col[0].W2.v[1], 1), rax = __shfl_down_sync(kAll, col[0].W3.v[1], 1);
        const R rby = __shfl_down_sync(kAll, col[0].W2.v[2], 1), ray = __shfl_down_sync(kAll, col[0].W3.v[2], 1);
        // column c0: c0-1 from the left lane, c0+1 = own second column
        viscous_add<1, R>(p, k, col[0].W3.v[0], col[0].W2.v[0], col[0].W3.v[1], col[0].W3.v[2], col[0].W2.v[1],
                          col[0].W2.v[2], col[1].W2.v[1] + col[1].W3.v[1], col[1].W2.v[2] + col[1].W3.v[2],
                          lbx + lax, lby + lay, Fy2[0]);
        // column c0+1: c0 = own first column, c0+2 from the right lane
        viscous_add<1, R>(p, k, col[1].W3.v[0], col[1].W2.v[0], col[1].W3.v[1], col[1].W3.v[2], col[1].W2.v[1],
                          col[1].W2.v[2], rbx + rax, rby + ray, col[0].W2.v[1] + col[0].W3.v[1],
                          col[0].W2.v[2] + col[0].W3.v[2], Fy2[1]);
      }
      if (tau) {
        const size_t rb = (size_t)wrap_fast(j - 2, p.ny) * p.nx, ra = (size_t)wrap_fast(j - 3, p.ny) * p.nx;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const R* tb = tau + (rb + gx[h]) * 3;
          const R* ta = tau + (ra + gx[h]) * 3;
          Fy2[h].v[1] = Fy2[h].v[1] + R(0.5) * (ta[1] + tb[1]);
          Fy2[h].v[2] = Fy2[h].v[2] + R(0.5) * (ta[2] + tb[2]);
        }
      }
    }
    if (it >= 6) {
      // ---- x sweep of row r = j-3 across the lanes -------------------------
      const int r = j - 3;
      const Cell4<R>& a = col[0].W3;
      const Cell4<R>& b = col[1].W3;
      const Cell4<R> La = shfl_up_cell<R, NV>(a, 1), Lb = shfl_up_cell<R, NV>(b, 1);
      const Cell4<R> Ra = shfl_down_cell<R, NV>(a, 1), Rb = shfl_down_cell<R, NV>(b, 1);
      Cell4<R> A0 = a, A1 = a, A2 = a;
      if constexpr (ReconTraits<RECON>::kFaceShared) {
        A0 = faces_cells<RECON, R, NV>(La, Lb, a, b);  // face c0 (between c0-1 and c0)
        A1 = faces_cells<RECON, R, NV>(Lb, a, b, Ra);  // face c0+1
        A2 = shfl_down_cell<R, NV>(A0, 1);             // face c0+2
      }
      Cell4<R> lo0, hi0, lo1, hi1;
      edges_cells<RECON, R, NV>(La, Lb, a, b, Ra, A0, A1, k.dfloor, lo0, hi0);
      edges_cells<RECON, R, NV>(Lb, a, b, Ra, Rb, A1, A2, k.dfloor, lo1, hi1);
      const Cell4<R> hiL = shfl_up_cell<R, NV>(hi1, 1);  // upper edge of column c0-1
      Cell4<R> F0 = face_flux_cells<RS, 0, R, NV>(hiL, lo0, gas);  // face c0
      Cell4<R> F1 = face_flux_cells<RS, 0, R, NV>(hi0, lo1, gas);  // face c0+1
      if (p.visc_on) {
        // Transverse y differences: rows r+1 (W2) and r-1 (W4) at the face's two columns.
        const Cell4<R>& u0 = col[0].W2;
        const Cell4<R>& u1 = col[1].W2;
        const Cell4<R>& d0 = col[0].W4;
        const Cell4<R>& d1 = col[1].W4;
        const R lux = __shfl_up_sync(kAll, u1.v[1], 1), luy = __shfl_up_sync(kAll, u1.v[2], 1);
        const R ldx = __shfl_up_sync(kAll, d1.v[1], 1), ldy = __shfl_up_sync(kAll, d1.v[2], 1);
        viscous_add<0, R>(p, k, Lb.v[0], a.v[0], Lb.v[1], Lb.v[2], a.v[1], a.v[2], u0.v[1] + lux, u0.v[2] + luy,
                          d0.v[1] + ldx, d0.v[2] + ldy, F0);
        viscous_add<0, R>(p, k, a.v[0], b.v[0], a.v[1], a.v[2], b.v[1], b.v[2], u1.v[1] + u0.v[1],
                          u1.v[2] + u0.v[2], d1.v[1] + d0.v[1], d1.v[2] + d0.v[2], F1);
      }
      if (tau) {
        const size_t rr = (size_t)wrap_fast(r, p.ny) * p.nx;
        const int gm = wrap_fast(c0 - 1, p.nx);
        const R* t0 = tau + (rr + gx[0]) * 3;
        const R* t1 = tau + (rr + gx[1]) * 3;
        const R* tm = tau + (rr + gm) * 3;
        F0.v[1] = F0.v[1] + R(0.5) * (tm[0] + t0[0]);
        F0.v[2] = F0.v[2] + R(0.5) * (tm[1] + t0[1]);
        F1.v[1] = F1.v[1] + R(0.5) * (t0[0] + t1[0]);
        F1.v[2] = F1.v[2] + R(0.5) * (t0[1] + t1[1]);
      }
      const Cell4<R> F2 = shfl_down_cell<R, NV>(F0, 1);  // face c0+2
      if (r < p.ny) {
        const size_t row = (size_t)r * p.nx;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!out[h]) continue;
          const size_t cell = row + (size_t)(c0 + h);
          const Cell4<R>& fl = h == 0 ? F0 : F1;
          const Cell4<R>& fr = h == 0 ? F1 : F2;
          const Cell4<R>& w = col[h].W3;
          Cell4<R> u = load_cell<R, NV>(U + cell * NV);
          u.v[0] = w.v[0];  // the floored density
          Cell4<R> vs = load_cell<R, NV>(V + cell * NV);
          if (p.floor_v) vs.v[0] = N::lt(vs.v[0], k.dfloor) ? k.dfloor : vs.v[0];
          Cell4<R> un;
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            if (p.has_delta) vs.v[v] = vs.v[v] + k.delta * u.v[v];
            un.v[v] = rk_combine<R>(p.blend, k.g0, k.g1, u.v[v], vs.v[v], fr.v[v] - fl.v[v],
                                    Fy2[h].v[v] - col[h].Fy3.v[v], ncx, ncy);
          }
          un.v[3] = NV == 4 ? un.v[3] : R(0);
          if (p.drag_on) {
            un.v[1] = un.v[1] + -((kdrag * w.v[0]) * w.v[1]);
            un.v[2] = un.v[2] + -((kdrag * w.v[0]) * w.v[2]);
          }
          if (p.has_delta && Vo) store_cell<R, NV>(Vo + cell * NV, vs);
          if (p.floor_out) un.v[0] = N::lt(un.v[0], k.dfloor) ? k.dfloor : un.v[0];
          store_cell<R, NV>(Uo + cell * NV, un);
          if (p.want_cfl) {
            const R inv = Num<R>::rcp(un.v[0]);
            vmax0 = N::nanmax_pos(vmax0, fabs(inv * un.v[1]) + k.cs);
            vmax1 = N::nanmax_pos(vmax1, fabs(inv * un.v[2]) + k.cs);
          }
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      col[h].Ay2 = Ay1[h];
      col[h].hy3 = hi[h];
      col[h].Fy3 = Fy2[h];
    }
  }
  if (p.want_cfl) {
    const double m0 = warp_nan_max(static_cast<double>(vmax0));
    const double m1 = warp_nan_max(static_cast<double>(vmax1));
    if (lane == 0) {
      p.partials[(size_t)tile * kCflSlots + 0] = m0;
      p.partials[(size_t)tile * kCflSlots + 1] = m1;
      p.partials[(size_t)tile * kCflSlots + 2] = 0.0;
      if (tile == 0) p.header->n_cfl = ntiles;
    }
  }
}

// Resident warps per SM the float32 kernels are compiled for, the most whose
// registers still hold every live value (no spills): for one solve, whose
// stage parameters sit in the constant bank, 16 (128 registers per thread)
// with DC/PLM/PPM4 and 12 with the longer PPMX/WENO-Z stencils; the batch
// kernel holds the parameters in registers and gets 12 and 8. The float64
// kernels use what they need.
template <typename R, int RECON> constexpr int march_min_blocks() {
  return sizeof(R) == 4 ? (RECON >= 3 ? 12 : 16) / kMarchWarps : 1;
}
template <typename R, int RECON> constexpr int march_batch_min_blocks() {
  return sizeof(R) == 4 ? (RECON >= 3 ? 8 : 12) / kMarchWarps : 1;
}

// One warp per tile; the block's warps take consecutive tiles.
template <typename R, int RECON, int RS, int NV>
__global__ void __launch_bounds__(kMarchWarps * 32, march_min_blocks<R, RECON>())
    stage_kernel_march(const StageParams p, int ntiles) {
  if (p.clock->done) return;
  const int tile = blockIdx.x * kMarchWarps + (threadIdx.x >> 5);
  if (tile >= ntiles) return;
  march_tile<R, RECON, RS, NV, false>(p, tile, ntiles);
}

// Persistent batch kernel over marching tiles (see stage_kernel_batch): each
// warp takes work items round-robin; nothing is shared between warps. A
// launch group holds solves of one variable count.
template <typename R, int RECON, int RS, int NV>
__global__ void __launch_bounds__(kMarchWarps * 32, march_batch_min_blocks<R, RECON>()) stage_kernel_batch_march(
    const StageParams* __restrict__ params, const int* __restrict__ tile_offset, int nsolves, int nwork) {
  const int stride = gridDim.x * kMarchWarps;
  for (int w = blockIdx.x * kMarchWarps + (threadIdx.x >> 5); w < nwork; w += stride) {
    int lo = 0, hi = nsolves - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile_offset[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const StageParams& p = params[lo];
    if (p.skip || p.clock->done) continue;
    const int tile = w - tile_offset[lo];
    march_tile<R, RECON, RS, NV, true>(p, tile, tile_offset[lo + 1] - tile_offset[lo]);
  }
}

// grid.x = number of tiles (one warp each).
template <typename R, int RECON, int RS, int NV>
cudaError_t launch_march_one(const StageParams& p, dim3 grid, cudaStream_t s) {
  const int ntiles = (int)grid.x;
  stage_kernel_march<R, RECON, RS, NV><<<(ntiles + kMarchWarps - 1) / kMarchWarps, kMarchWarps * 32, 0, s>>>(p, ntiles);
  return cudaGetLastError();
}

template <typename R, int RECON>
cudaError_t launch_march_typed(int rsolver, const StageParams& p, dim3 grid, cudaStream_t s) {
  const bool three = p.nv == 3;
  switch (rsolver) {
    case JX_LLF: return three ? launch_march_one<R, RECON, JX_LLF, 3>(p, grid, s) : launch_march_one<R, RECON, JX_LLF, 4>(p, grid, s);
    case JX_HLLE: return three ? launch_march_one<R, RECON, JX_HLLE, 3>(p, grid, s) : launch_march_one<R, RECON, JX_HLLE, 4>(p, grid, s);
    case JX_ROE: return three ? launch_march_one<R, RECON, JX_ROE, 3>(p, grid, s) : launch_march_one<R, RECON, JX_ROE, 4>(p, grid, s);
  }
  return cudaErrorInvalidValue;
}

template <typename R, int RECON, int NV>
cudaError_t launch_batch_march_nv(int rsolver, const StageParams* params, const int* offsets, int nsolves,
                                  int nwork, dim3 grid, cudaStream_t s) {
  constexpr int T = kMarchWarps * 32;
  switch (rsolver) {
    case JX_LLF: stage_kernel_batch_march<R, RECON, JX_LLF, NV><<<grid, T, 0, s>>>(params, offsets, nsolves, nwork); break;
    case JX_HLLE: stage_kernel_batch_march<R, RECON, JX_HLLE, NV><<<grid, T, 0, s>>>(params, offsets, nsolves, nwork); break;
    case JX_ROE: stage_kernel_batch_march<R, RECON, JX_ROE, NV><<<grid, T, 0, s>>>(params, offsets, nsolves, nwork); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename R, int RECON>
cudaError_t launch_batch_march_typed(int rsolver, int nv, const StageParams* params, const int* offsets,
                                     int nsolves, int nwork, dim3 grid, cudaStream_t s) {
  return nv == 3 ? launch_batch_march_nv<R, RECON, 3>(rsolver, params, offsets, nsolves, nwork, grid, s)
                 : launch_batch_march_nv<R, RECON, 4>(rsolver, params, offsets, nsolves, nwork, grid, s);
}

}  // namespace jx

namespace jx {

template <int RECON>
cudaError_t launch_march_recon(int dtype, int rsolver, const StageParams& p, dim3 grid, cudaStream_t s) {
  if (dtype == JX_F64) return launch_march_typed<double, RECON>(rsolver, p, grid, s);
  return launch_march_typed<float, RECON>(rsolver, p, grid, s);
}

template <int RECON>
cudaError_t launch_batch_march_recon(int dtype, int rsolver, int nv, const StageParams* params, const int* offsets,
                                     int nsolves, int nwork, dim3 grid, cudaStream_t s) {
  if (dtype == JX_F64)
    return launch_batch_march_typed<double, RECON>(rsolver, nv, params, offsets, nsolves, nwork, grid, s);
  return launch_batch_march_typed<float, RECON>(rsolver, nv, params, offsets, nsolves, nwork, grid, s);
}

template <typename Kernel>
int march_occupancy(Kernel kernel) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kMarchWarps * 32, 0) != cudaSuccess) return 0;
  return n;
}

// Resident marching blocks per SM (single-solve or batch kernel).
template <typename R, int RECON, int RS>
int march_blocks_per_sm_rs(int nv, bool batch) {
  if (batch)
    return nv == 3 ? march_occupancy(stage_kernel_batch_march<R, RECON, RS, 3>)
                   : march_occupancy(stage_kernel_batch_march<R, RECON, RS, 4>);
  return nv == 3 ? march_occupancy(stage_kernel_march<R, RECON, RS, 3>)
                 : march_occupancy(stage_kernel_march<R, RECON, RS, 4>);
}

template <int RECON>
int march_blocks_per_sm_recon(int dtype, int rsolver, int nv, bool batch) {
  if (dtype == JX_F64) {
    if (rsolver == JX_LLF) return march_blocks_per_sm_rs<double, RECON, JX_LLF>(nv, batch);
    if (rsolver == JX_HLLE) return march_blocks_per_sm_rs<double, RECON, JX_HLLE>(nv, batch);
    return march_blocks_per_sm_rs<double, RECON, JX_ROE>(nv, batch);
  }
  if (rsolver == JX_LLF) return march_blocks_per_sm_rs<float, RECON, JX_LLF>(nv, batch);
  if (rsolver == JX_HLLE) return march_blocks_per_sm_rs<float, RECON, JX_HLLE>(nv, batch);
  return march_blocks_per_sm_rs<float, RECON, JX_ROE>(nv, batch);
}

}  // namespace jx
