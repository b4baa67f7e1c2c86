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
// There is no barrier and no data shared between lanes through memory (on
// float32 tiles of 24 rows or more each lane stages its own rows in a
// shared-memory ring, see kRingU); a warp's CFL partial (the exact maximum
// over its tile) goes to the workspace slot of its tile. Arithmetic
// per cell is the same as in jx_stage_fast.cuh (same device functions in the
// same order), so results agree with it to rounding.
#pragma once
#include "jx_device.cuh"
#include "jx_internal.h"
#include "jx_stage_fast.cuh"
#include "jx_ring.cuh"
#include "jx_stage_march_pk.cuh"

#include <utility>

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
  for (int v = 1; v < 4; ++v) w.v[v] = v < NV ? Ops<R>::mul(inv, u.v[v]) : R(0);
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
  for (int v = 3; v < NV; ++v) f.v[v] = scalar_flux(f0, L.v[v], Rv.v[v]);
  return f;
}

// Viscous momentum flux at a face (fluxes.py:227-266) from the velocities of
// the two cells a (low side) and b (high side) and the transverse difference
// ((b+ + a+) - (b- + a-)); rho_a, rho_b their densities.
template <int DIR, typename R>
__device__ __forceinline__ void viscous_add(const StageParams& p, const StageConsts<R>& k, R rho_a, R rho_b,
                                            R ax, R ay, R bx, R by, R tpx, R tpy, R tmx, R tmy, Cell4<R>& f) {
  viscous_face<DIR, R>(p.smag_on, k.nu, k.smag_c, DIR == 0 ? k.inv_dx : k.inv_dy, DIR == 0 ? k.inv_4dy : k.inv_4dx,
                       rho_a, rho_b, ax, ay, bx, by, tpx, tpy, tmx, tmy, f.v[1], f.v[2]);
}

// One column of a lane: a 5-row window of primitives (rows j-4 .. j), the
// face value below row j-1, the upper edge of row j-3 and the y flux below
// row j-3 (see the file comment).
template <typename R> struct MarchColumn {
  Cell4<R> W4, W3, W2, W1, W0, Ay2, hy3, Fy3;
};


// The cell at column c0 + K of the lane's row, K in [-2, NC + 1]: one of
// the lane's own NC columns, or a neighbouring lane's by a warp shuffle.
template <int K, int NC, typename R, int NV>
__device__ __forceinline__ Cell4<R> lane_cell(const Cell4<R> (&own)[NC]) {
  if constexpr (K >= 0 && K < NC) {
    return own[K];
  } else if constexpr (K < 0) {
    constexpr int back = (-K + NC - 1) / NC;
    return shfl_up_cell<R, NV>(own[K + back * NC], back);
  } else {
    constexpr int ahead = K / NC;
    return shfl_down_cell<R, NV>(own[K - ahead * NC], ahead);
  }
}

template <int NC, typename R, int NV, int... I>
__device__ __forceinline__ void lane_cells_impl(const Cell4<R> (&own)[NC], Cell4<R> (&E)[NC + 4],
                                                std::integer_sequence<int, I...>) {
  ((E[I] = lane_cell<I - 2, NC, R, NV>(own)), ...);
}

// E[k + 2] = the cell at column c0 + k, k = -2 .. NC + 1.
template <int NC, typename R, int NV>
__device__ __forceinline__ void lane_cells(const Cell4<R> (&own)[NC], Cell4<R> (&E)[NC + 4]) {
  lane_cells_impl<NC, R, NV>(own, E, std::make_integer_sequence<int, NC + 4>{});
}


// PREFETCH_V: issue L2 prefetches of the saved register two rows ahead of
// the RK combine. Measured on GB300: it helps the batch kernel (12 resident
// warps per SM, ensemble cycle -2.2 %) and costs the single-solve kernel
// (16 warps, already hiding the latency; +2.4 % at 4096²). Results do not
// depend on it.
//
// NC columns per lane: lane l holds columns c0 .. c0 + NC - 1 of a strip of
// 32 NC columns (c0 = x0 - 3 + NC l), of which the middle 32 NC - 6 are the
// tile's outputs. Every cell's arithmetic is the same whatever NC is, so
// results do not depend on it.
//
// The walk is a 6-row prologue (the rows above the tile's first output row
// only feed the y sweep) and a steady loop in which every phase runs and no
// phase is tested. The steady loop is deliberately not unrolled: unrolling it
// by 2, 3 or 5 (so that the register window would shift by renaming instead
// of moves) measured 5, 12 and 34 % slower on GB300, the body outgrowing the
// instruction cache. Lanes whose columns are ghosts (or beyond a ragged right
// edge) run the RK combine on a cell of their own tile and skip only the
// store, so the combine has no divergent branch.
template <typename R, int RECON, int RS, int NV, int NC, int FORM, bool PREFETCH_V, bool RING = false>
__device__ __forceinline__ void march_tile(const StageParams& p, int tile, int ntiles, float4* ring = nullptr) {
  using N = Num<R>;
  constexpr bool kLean = FORM != kMarchGeneric;
  constexpr int TX = march_tile_x(NC);
  const StageConsts<R>& k = stage_consts<R>(p);
  const int lane = threadIdx.x & 31;
  const int TY = p.ty;
  const int bx = tile % p.tiles_x, by = tile / p.tiles_x;
  const int x0 = bx * TX;  // first output column of the tile
  const int y0 = by * TY;
  const int c0 = x0 - 3 + NC * lane;  // this lane's columns: c0 .. c0 + NC - 1
  const int xlast = min(x0 + TX, p.nx) - 1;
  int gx[NC], cx[NC];
  bool out[NC];
#pragma unroll
  for (int h = 0; h < NC; ++h) {
    gx[h] = wrap_fast(c0 + h, p.nx);
    // Local columns 3 .. 32 NC - 4 of the strip are written.
    const int local = NC * lane + h;
    out[h] = local >= 3 && local <= 32 * NC - 4 && c0 + h < p.nx;
    // Column of the RK combine's loads: the lane's own for written cells,
    // else the nearest written column of the tile (same cache lines, no
    // divergence).
    cx[h] = min(max(c0 + h, x0), xlast);
  }
  const R* __restrict__ U = static_cast<const R*>(p.U);
  const R* __restrict__ V = static_cast<const R*>(p.V);
  R* Uo = static_cast<R*>(p.Uout);
  R* Vo = static_cast<R*>(p.Vout);
  const R* __restrict__ tau = kLean ? nullptr : static_cast<const R*>(p.tau);
  const bool visc = !kLean && p.visc_on;
  const bool drag = !kLean && p.drag_on;
  const bool blend = kLean ? FORM == kMarchLeanBlend : (bool)p.blend;
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

  MarchColumn<R> col[NC];
#pragma unroll
  for (int h = 0; h < NC; ++h) col[h].W4 = col[h].W3 = col[h].W2 = col[h].W1 = col[h].W0 = col[h].Ay2 =
      col[h].hy3 = col[h].Fy3 = Cell4<R>{};
  R vmax0 = R(0), vmax1 = R(0);
  const int iters = TY + 6;
  Cell4<R> next[NC];
  // Ring slots of this lane: U row t (t = it) at ringU(t, h), V at ringV(t, h).
  auto ringU = [&](int t, int h) { return ring + ((t & (kRingU - 1)) * NC + h) * 32 + lane; };
  auto ringV = [&](int t, int h) { return ring + (kRingU * NC + (t & (kRingV - 1)) * NC + h) * 32 + lane; };
  if constexpr (RING) {
    for (int t = 0; t < kRingAhead; ++t) {
      const size_t row = (size_t)wrap_fast(y0 - 3 + t, p.ny) * p.nx;
#pragma unroll
      for (int h = 0; h < NC; ++h) ring_copy<NV>(ringU(t, h), U + (row + gx[h]) * NV);
      cp_async_commit();
    }
  } else {
    const size_t row = (size_t)wrap_fast(y0 - 3, p.ny) * p.nx;
#pragma unroll
    for (int h = 0; h < NC; ++h) next[h] = load_cell<R, NV>(U + (row + gx[h]) * NV);
  }
  // One row of the walk: row j = y0 - 3 + it arrives. STEADY: it >= 6.
  auto walk_row = [&](const int it, auto steady_tag) {
    constexpr bool kSteady = decltype(steady_tag)::value;
    const int j = y0 - 3 + it;
    // ---- y sweep of every column -------------------------------------------
    Cell4<R> Ay1[NC], lo[NC], hi[NC], Fy2[NC];
    if constexpr (RING) {
      // kRingAhead + it groups are committed: the prologue's kRingAhead
      // (U rows 0 .. kRingAhead - 1) and one per earlier row. This row's U
      // and the V the combine reads below (row it - 3) came in group it,
      // so all but the kRingAhead - 1 newest groups must have landed.
      cp_async_wait<kRingAhead - 1>();
#pragma unroll
      for (int h = 0; h < NC; ++h) next[h] = ring_read<NV>(ringU(it, h));
    }
#pragma unroll
    for (int h = 0; h < NC; ++h) {
      MarchColumn<R>& c = col[h];
      c.W4 = c.W3;
      c.W3 = c.W2;
      c.W2 = c.W1;
      c.W1 = c.W0;
      c.W0 = recover_cell<R, NV>(next[h], k.dfloor);
    }
    if constexpr (RING) {
      // U row it + 3 (only rows the walk reaches) and V of row it (a tile
      // row the combine will update, three iterations from now).
      if (it + kRingAhead < iters) {
        const size_t row = (size_t)wrap_fast(j + kRingAhead, p.ny) * p.nx;
#pragma unroll
        for (int h = 0; h < NC; ++h) ring_copy<NV>(ringU(it + kRingAhead, h), U + (row + gx[h]) * NV);
      }
      if (it >= 3 && j < p.ny && it < TY + 3) {
        const size_t row = (size_t)j * p.nx;
#pragma unroll
        for (int h = 0; h < NC; ++h) ring_copy<NV>(ringV(it, h), V + (row + (size_t)cx[h]) * NV);
      }
      cp_async_commit();
    } else {
      // The row after this one (past the tile's last row: a wrapped row
      // that is never used, cheaper than a test).
      const size_t row = (size_t)wrap_fast(j + 1, p.ny) * p.nx;
#pragma unroll
      for (int h = 0; h < NC; ++h) next[h] = load_cell<R, NV>(U + (row + gx[h]) * NV);
    }
    // The saved register V is read once, by the RK combine of row j-3; ask L2
    // for row j-1 now (two rows ahead, no registers held) so that the combine
    // does not wait for DRAM. Only cells the combine will read.
    if (PREFETCH_V && (kSteady || it >= 4) && j - 1 < p.ny && j - 1 < y0 + TY) {
      const size_t row = (size_t)(j - 1) * p.nx;
#pragma unroll
      for (int h = 0; h < NC; ++h)
        if (out[h]) asm volatile("prefetch.global.L2 [%0];" ::"l"(V + (row + (size_t)(c0 + h)) * NV));
    }
#pragma unroll
    for (int h = 0; h < NC; ++h) {
      MarchColumn<R>& c = col[h];
      Ay1[h] = c.Ay2;
      if ((kSteady || it >= 3) && ReconTraits<RECON>::kFaceShared) Ay1[h] = faces_cells<RECON, R, NV>(c.W3, c.W2, c.W1, c.W0);
      hi[h] = c.hy3;
      lo[h] = c.hy3;
      if (kSteady || it >= 4) edges_cells<RECON, R, NV>(c.W4, c.W3, c.W2, c.W1, c.W0, c.Ay2, Ay1[h], k.dfloor, lo[h], hi[h]);
      Fy2[h] = c.Fy3;
    }
    if (kSteady || it >= 5) {
      // Faces between rows j-3 (a) and j-2 (b).
#pragma unroll
      for (int h = 0; h < NC; ++h) Fy2[h] = face_flux_cells<RS, 1, R, NV>(col[h].hy3, lo[h], gas);
      if (visc) {
        // Transverse x differences: (row j-2 + row j-3) at columns h+1 and h-1.
        R sx[NC + 2], sy[NC + 2];  // sx[h + 1]: column h, h = -1 .. NC
#pragma unroll
        for (int h = 0; h < NC; ++h) {
          sx[h + 1] = col[h].W2.v[1] + col[h].W3.v[1];
          sy[h + 1] = col[h].W2.v[2] + col[h].W3.v[2];
        }
        // The neighbours' sums are formed from shuffled addends, in the same
        // order, so every column's sum is the same number.
        sx[0] = __shfl_up_sync(kAll, col[NC - 1].W2.v[1], 1) + __shfl_up_sync(kAll, col[NC - 1].W3.v[1], 1);
        sy[0] = __shfl_up_sync(kAll, col[NC - 1].W2.v[2], 1) + __shfl_up_sync(kAll, col[NC - 1].W3.v[2], 1);
        sx[NC + 1] = __shfl_down_sync(kAll, col[0].W2.v[1], 1) + __shfl_down_sync(kAll, col[0].W3.v[1], 1);
        sy[NC + 1] = __shfl_down_sync(kAll, col[0].W2.v[2], 1) + __shfl_down_sync(kAll, col[0].W3.v[2], 1);
#pragma unroll
        for (int h = 0; h < NC; ++h)
          viscous_add<1, R>(p, k, col[h].W3.v[0], col[h].W2.v[0], col[h].W3.v[1], col[h].W3.v[2], col[h].W2.v[1],
                            col[h].W2.v[2], sx[h + 2], sy[h + 2], sx[h], sy[h], Fy2[h]);
      }
      if (tau) {
        const size_t rb = (size_t)wrap_fast(j - 2, p.ny) * p.nx, ra = (size_t)wrap_fast(j - 3, p.ny) * p.nx;
#pragma unroll
        for (int h = 0; h < NC; ++h) {
          const R* tb = tau + (rb + gx[h]) * 3;
          const R* ta = tau + (ra + gx[h]) * 3;
          Fy2[h].v[1] = add_half_sum(Fy2[h].v[1], ta[1], tb[1]);
          Fy2[h].v[2] = add_half_sum(Fy2[h].v[2], ta[2], tb[2]);
        }
      }
    }
    if (kSteady) {
      // ---- x sweep of row r = j-3 across the lanes -------------------------
      const int r = j - 3;
      Cell4<R> own[NC];
#pragma unroll
      for (int h = 0; h < NC; ++h) own[h] = col[h].W3;
      Cell4<R> E[NC + 4];  // E[k + 2]: column c0 + k
      lane_cells<NC, R, NV>(own, E);
      Cell4<R> A[NC + 1];  // A[h]: face between columns h-1 and h
#pragma unroll
      for (int h = 0; h <= NC; ++h) A[h] = E[2];
      if constexpr (ReconTraits<RECON>::kFaceShared) {
#pragma unroll
        for (int h = 0; h < NC; ++h) A[h] = faces_cells<RECON, R, NV>(E[h], E[h + 1], E[h + 2], E[h + 3]);
        A[NC] = shfl_down_cell<R, NV>(A[0], 1);
      }
      Cell4<R> lx[NC], hx[NC];
#pragma unroll
      for (int h = 0; h < NC; ++h)
        edges_cells<RECON, R, NV>(E[h], E[h + 1], E[h + 2], E[h + 3], E[h + 4], A[h], A[h + 1], k.dfloor, lx[h], hx[h]);
      const Cell4<R> hiL = shfl_up_cell<R, NV>(hx[NC - 1], 1);  // upper edge of column c0-1
      Cell4<R> F[NC + 1];  // F[h]: flux at face h
#pragma unroll
      for (int h = 0; h < NC; ++h) F[h] = face_flux_cells<RS, 0, R, NV>(h == 0 ? hiL : hx[h - 1], lx[h], gas);
      if (visc) {
        // Transverse y differences: rows r+1 (W2) and r-1 (W4) at the face's two columns.
        R ux[NC + 1], uy[NC + 1], dx[NC + 1], dy[NC + 1];  // [h + 1]: column h, h = -1 .. NC-1
#pragma unroll
        for (int h = 0; h < NC; ++h) {
          ux[h + 1] = col[h].W2.v[1];
          uy[h + 1] = col[h].W2.v[2];
          dx[h + 1] = col[h].W4.v[1];
          dy[h + 1] = col[h].W4.v[2];
        }
        ux[0] = __shfl_up_sync(kAll, col[NC - 1].W2.v[1], 1);
        uy[0] = __shfl_up_sync(kAll, col[NC - 1].W2.v[2], 1);
        dx[0] = __shfl_up_sync(kAll, col[NC - 1].W4.v[1], 1);
        dy[0] = __shfl_up_sync(kAll, col[NC - 1].W4.v[2], 1);
#pragma unroll
        for (int h = 0; h < NC; ++h) {
          const Cell4<R>& a = E[h + 1];  // column h-1
          const Cell4<R>& b = E[h + 2];  // column h
          viscous_add<0, R>(p, k, a.v[0], b.v[0], a.v[1], a.v[2], b.v[1], b.v[2], ux[h + 1] + ux[h], uy[h + 1] + uy[h],
                            dx[h + 1] + dx[h], dy[h + 1] + dy[h], F[h]);
        }
      }
      if (tau) {
        const size_t rr = (size_t)wrap_fast(r, p.ny) * p.nx;
        const int gm = wrap_fast(c0 - 1, p.nx);
#pragma unroll
        for (int h = 0; h < NC; ++h) {
          const R* ta = tau + (rr + (h == 0 ? gm : gx[h - 1])) * 3;
          const R* tb = tau + (rr + gx[h]) * 3;
          F[h].v[1] = add_half_sum(F[h].v[1], ta[0], tb[0]);
          F[h].v[2] = add_half_sum(F[h].v[2], ta[1], tb[1]);
        }
      }
      F[NC] = shfl_down_cell<R, NV>(F[0], 1);  // face c0 + NC
      if (r < p.ny) {
        const size_t row = (size_t)r * p.nx;
#pragma unroll
        for (int h = 0; h < NC; ++h) {
          const size_t cell = row + (size_t)cx[h];
          const Cell4<R>& fl = F[h];
          const Cell4<R>& fr = F[h + 1];
          const Cell4<R>& w = col[h].W3;
          Cell4<R> u, vs;
          if constexpr (RING) {
            // Row r is walk row it - 3: its U is still in the ring (for a
            // ghost lane that is the lane's own column, not cx: the result
            // is not stored), its V landed with this row's group.
            u = ring_read<NV>(ringU(it - 3, h));
            vs = ring_read<NV>(ringV(it - 3, h));
          } else {
            u = load_cell<R, NV>(U + cell * NV);
            vs = load_cell<R, NV>(V + cell * NV);
          }
          u.v[0] = w.v[0];  // the floored density
          if (p.floor_v) vs.v[0] = N::lt(vs.v[0], k.dfloor) ? k.dfloor : vs.v[0];
          Cell4<R> un;
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            if (p.has_delta) vs.v[v] = delta_update(vs.v[v], k.delta, u.v[v]);
            // The flux differences round on their own: a flux held in this
            // thread's registers (not read back from another lane) must not be
            // fused into the difference.
            un.v[v] = rk_combine<R>(blend, k.g0, k.g1, u.v[v], vs.v[v], Ops<R>::sub(fr.v[v], fl.v[v]),
                                    Ops<R>::sub(Fy2[h].v[v], col[h].Fy3.v[v]), ncx, ncy);
          }
          un.v[3] = NV == 4 ? un.v[3] : R(0);
          if (drag) {
            un.v[1] = drag_term(un.v[1], kdrag * w.v[0], w.v[1]);
            un.v[2] = drag_term(un.v[2], kdrag * w.v[0], w.v[2]);
          }
          if (p.floor_out) un.v[0] = N::lt(un.v[0], k.dfloor) ? k.dfloor : un.v[0];
          if (out[h]) {
            if (p.has_delta && Vo) store_cell<R, NV>(Vo + cell * NV, vs);
            store_cell<R, NV>(Uo + cell * NV, un);
          }
          if (p.want_cfl) {
            const R inv = Num<R>::rcp(un.v[0]);
            const R s0 = signal_speed(inv, un.v[1], k.cs), s1 = signal_speed(inv, un.v[2], k.cs);
            if (out[h]) {
              vmax0 = N::nanmax_pos(vmax0, s0);
              vmax1 = N::nanmax_pos(vmax1, s1);
            }
          }
        }
      }
    }
#pragma unroll
    for (int h = 0; h < NC; ++h) {
      col[h].Ay2 = Ay1[h];
      col[h].hy3 = hi[h];
      col[h].Fy3 = Fy2[h];
    }
  };
  for (int it = 0; it < 6; ++it) walk_row(it, Flag<false>{});
#pragma unroll 1
  for (int it = 6; it < iters; ++it) walk_row(it, Flag<true>{});
  if constexpr (RING) cp_async_wait_all();
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

// The form a stage runs in (see MarchForm).
__host__ __device__ inline int march_form(const StageParams& p) {
  if (p.visc_on || p.tau || p.drag_on) return kMarchGeneric;
  return p.blend ? kMarchLeanBlend : kMarchLeanPlain;
}

// Resident warps per SM the kernels are compiled for (the register cap),
// chosen so that every live value stays in registers (no spills): for one
// float32 solve, whose stage parameters sit in the constant bank, 16 warps
// (128 registers per thread) with two columns per lane and DC/PLM/PPM4, 12
// with the longer PPMX/WENO-Z stencils; one column per lane needs fewer
// registers (24 / 16 warps), three need more (12 / 8). The batch kernel holds
// the parameters in registers and gets 4 warps fewer. Float64 uses what it
// needs.
template <typename R, int RECON, int NC> constexpr int march_min_blocks() {
  if constexpr (sizeof(R) != 4) return 1;
  const int two = RECON >= 3 ? 12 : 16;
  return (NC == 1 ? two + (RECON >= 3 ? 4 : 8) : (NC == 3 ? two - 4 : two)) / kMarchWarps;
}
template <typename R, int RECON, int NC> constexpr int march_batch_min_blocks() {
  return sizeof(R) == 4 ? march_min_blocks<R, RECON, NC>() - 4 / kMarchWarps : 1;
}

// One warp per tile; the block's warps take consecutive tiles.
// RING (float32 only): the row ring above, march_smem bytes of dynamic
// shared memory per block.
template <typename R, int RECON, int RS, int NV, int NC, int FORM, bool RING = false>
__global__ void __launch_bounds__(kMarchWarps * 32, (march_min_blocks<R, RECON, NC>()))
    stage_kernel_march(const StageParams p, int ntiles) {
  if (p.clock->done) return;
  const int tile = blockIdx.x * kMarchWarps + (threadIdx.x >> 5);
  if (tile >= ntiles) return;
  if constexpr (RING && sizeof(R) == 4) {
    extern __shared__ float4 march_ring[];
    march_tile<R, RECON, RS, NV, NC, FORM, false, true>(p, tile, ntiles,
                                                       march_ring + (threadIdx.x >> 5) * (march_ring_bytes<NC>() / 16));
  } else {
    march_tile<R, RECON, RS, NV, NC, FORM, false>(p, tile, ntiles);
  }
}

template <int NC> constexpr size_t march_smem() { return (size_t)march_ring_bytes<NC>() * kMarchWarps; }

// PLM, PPM4, PPMX and WENO-Z with two columns per lane run the packed-pair
// walk of jx_stage_march_pk.cuh (float32) where it measured faster than the
// per-column walk (GB300, RK3 stage 2): 4 variables in the lean forms and 3
// in the generic form.
//   * PPM4/Roe 0.2812 -> 0.2642 ms at 4096² (58 x 121, with the row ring),
//     0.0269 -> 0.0249 ms at 1024² (58 x 8); HLLE 0.2886 -> 0.2717 and
//     0.0270 -> 0.0250 ms; LLF 0.0221 -> 0.0208 ms at 1024², but its ring
//     kernel spills (0.2437 -> 0.2618 ms), so LLF's tall tiles keep the
//     per-column ring walk;
//   * PLM/HLLE 0.3466 -> 0.3259 ms at 4096², 0.0311 -> 0.0290 ms at 1024²;
//   * PPMX/Roe 0.6559 -> 0.6014 and 0.0577 -> 0.0535 ms; LLF 0.5699 ->
//     0.5467 and 0.0518 -> 0.0496 ms;
//   * WENO-Z/HLLE on 58 x 121 tiles 1.481 -> 1.344 ms, but on the 8-row
//     tiles of a 1024² grid 0.123 -> 0.156 ms, so only tall tiles use it
//     (WENO-Z defaults to one column per lane, which it does not cover);
//   * DC: 0.176 -> 0.202 ms at 4096², 0.0144 ms either way at 1024²: not used;
//   * 3 variables, lean: PPM4 1 % slower (0.2379 -> 0.2404 ms): not used;
//     3 variables, generic form (viscosity and drag): PPM4/Roe 0.2944 ->
//     0.2704 ms at 4096², 0.0270 -> 0.0249 ms at 1024², PLM/HLLE 0.3597 ->
//     0.3262 ms: used (not with SGS stress, which has no packed path);
//   * 4 variables, generic form: the kernel spills at 16 warps; not used.
template <typename R, int RECON, int RS, int NV, int NC, int FORM> constexpr bool march_packed() {
  return sizeof(R) == 4 && RECON != JX_DC && NC == 2 && (NV == 4 ? FORM != kMarchGeneric : FORM == kMarchGeneric);
}
template <int RECON> constexpr bool march_packed_short() { return RECON != JX_WENOZ; }
template <int RECON, int RS> constexpr bool march_packed_ring() { return RECON != JX_PPM4 || RS != JX_LLF; }

static_assert(kMarchWarps == 1, "the packed-pair kernel takes one tile per single-warp block");
template <int RECON, int RS, int NV, int FORM, bool RING>
__global__ void __launch_bounds__(32, RECON >= JX_PPMX ? 12 : 16) stage_kernel_march_pk(const StageParams p, int ntiles) {
  if (p.clock->done) return;
  const int tile = blockIdx.x;
  if (tile >= ntiles) return;
  extern __shared__ float4 march_ring[];
  pk::march_tile_pk<RECON, RS, NV, FORM, RING>(p, tile, ntiles, RING ? march_ring : nullptr);
}

// The PPM4 packed walk with the row ring, built at 112 registers with each
// row's x sweep ahead of its y sweep (XFIRST), which is what lets 112 fit
// without spills (the y sweep first spilled 20 bytes at 112 and took 0.328
// ms). Measured at 4096²: 0.2569-0.2589 ms per stage against 0.2645 ms for
// the y-first walk at 122 registers, the same bits; ncu at 3072² shows the
// same 16 resident blocks per SM (registers are allocated per scheduler, 16 K
// each: 112 or 122 a thread both leave room for 4 warps, 5 need 96 or fewer,
// which spills), the same instructions per cell, and issue 69.2 % of cycles
// against 67.3 %: the gain is the schedule, not occupancy. The x
// sweep first at 122 registers changed nothing, and short tiles (no ring)
// spill at 112. The register count is a template argument because nvcc
// accepts __launch_bounds__ beside __maxnreg__ only in that form (without
// the 32-thread block bound, 112 registers spill 8 bytes).
template <int RS, int NV, int FORM, int REGS = 112>
__global__ void __launch_bounds__(32) __maxnreg__(REGS) stage_kernel_march_pk_x(const StageParams p, int ntiles) {
  if (p.clock->done) return;
  const int tile = blockIdx.x;
  if (tile >= ntiles) return;
  extern __shared__ float4 march_ring[];
  pk::march_tile_pk<JX_PPM4, RS, NV, FORM, true, true>(p, tile, ntiles, march_ring);
}

// Let a ring kernel have the largest shared-memory carve-out (once per kernel).
template <auto Kernel>
void march_prefer_shared() {
  static const bool done = [] {
    cudaFuncSetAttribute(Kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaGetLastError();
    return true;
  }();
  (void)done;
}

// Persistent batch kernel over marching tiles (see stage_kernel_batch): each
// warp takes work items round-robin; nothing is shared between warps. A
// launch group holds solves of one variable count and one column count per
// lane; each solve's stage options are read at run time.
template <typename R, int RECON, int RS, int NV, int NC, bool RING = false>
__global__ void __launch_bounds__(kMarchWarps * 32, (march_batch_min_blocks<R, RECON, NC>())) stage_kernel_batch_march(
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
    if constexpr (RING && sizeof(R) == 4) {
      // The ring is free again at the end of each tile (march_tile waits for its copies).
      extern __shared__ float4 march_ring[];
      march_tile<R, RECON, RS, NV, NC, kMarchGeneric, false, true>(
          p, tile, tile_offset[lo + 1] - tile_offset[lo], march_ring + (threadIdx.x >> 5) * (march_ring_bytes<NC>() / 16));
    } else {
      march_tile<R, RECON, RS, NV, NC, kMarchGeneric, true>(p, tile, tile_offset[lo + 1] - tile_offset[lo]);
    }
  }
}

// Float32 stages run in their lean form when they have one; float64 (used
// only on request: its default is the shared-memory tile) always runs the
// generic form with two columns per lane. One column per lane (a latency
// choice for small grids) runs the generic form.
// Batched packed-pair walk (see stage_kernel_batch_march): a launch group of
// 4-variable lean solves with one integrator, so that every member's stage
// has the same form, or of 3-variable solves in the generic form.
template <int RECON, int RS, int NV, int FORM, bool RING>
__global__ void __launch_bounds__(32, RECON >= JX_PPMX ? 8 : 12) stage_kernel_batch_march_pk(
    const StageParams* __restrict__ params, const int* __restrict__ tile_offset, int nsolves, int nwork) {
  extern __shared__ float4 march_ring[];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    int lo = 0, hi = nsolves - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile_offset[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const StageParams& p = params[lo];
    if (p.skip || p.clock->done) continue;
    pk::march_tile_pk<RECON, RS, NV, FORM, RING>(p, w - tile_offset[lo],
                                                                   tile_offset[lo + 1] - tile_offset[lo],
                                                                   RING ? march_ring : nullptr);
  }
}

template <typename R, int RECON, int RS, int NV, int NC, int FORM>
cudaError_t launch_march_form(const StageParams& p, dim3 blocks, dim3 threads, int ntiles, cudaStream_t s) {
  if constexpr (march_packed<R, RECON, RS, NV, NC, FORM>()) {
    if (FORM == kMarchGeneric && p.tau) {
      // SGS stress: the per-column walk (the packed one has no stress path).
    } else if (p.ty < kRingMinRows) {
      if constexpr (march_packed_short<RECON>()) {
        stage_kernel_march_pk<RECON, RS, NV, FORM, false><<<blocks, threads, 0, s>>>(p, ntiles);
        return cudaGetLastError();
      }
    } else if constexpr (march_packed_ring<RECON, RS>()) {
      if constexpr (RECON == JX_PPM4) {
        march_prefer_shared<stage_kernel_march_pk_x<RS, NV, FORM>>();
        stage_kernel_march_pk_x<RS, NV, FORM><<<blocks, threads, march_smem<2>(), s>>>(p, ntiles);
      } else {
        march_prefer_shared<stage_kernel_march_pk<RECON, RS, NV, FORM, true>>();
        stage_kernel_march_pk<RECON, RS, NV, FORM, true><<<blocks, threads, march_smem<2>(), s>>>(p, ntiles);
      }
      return cudaGetLastError();
    }
  }
  if constexpr (march_ring_on<R, RECON, NC>()) {
    if (p.ty >= kRingMinRows) {
      march_prefer_shared<stage_kernel_march<R, RECON, RS, NV, NC, FORM, true>>();
      stage_kernel_march<R, RECON, RS, NV, NC, FORM, true><<<blocks, threads, march_smem<NC>(), s>>>(p, ntiles);
      return cudaGetLastError();
    }
  }
  stage_kernel_march<R, RECON, RS, NV, NC, FORM><<<blocks, threads, 0, s>>>(p, ntiles);
  return cudaGetLastError();
}

template <typename R, int RECON, int RS, int NV, int NC>
cudaError_t launch_march_nc(const StageParams& p, dim3 blocks, dim3 threads, int ntiles, cudaStream_t s) {
  if constexpr (sizeof(R) == 4 && NC > 1) {
    const int form = march_form(p);
    if (form == kMarchLeanBlend) return launch_march_form<R, RECON, RS, NV, NC, kMarchLeanBlend>(p, blocks, threads, ntiles, s);
    if (form == kMarchLeanPlain) return launch_march_form<R, RECON, RS, NV, NC, kMarchLeanPlain>(p, blocks, threads, ntiles, s);
  }
  return launch_march_form<R, RECON, RS, NV, NC, kMarchGeneric>(p, blocks, threads, ntiles, s);
}

// grid.x = number of tiles (one warp each); p.nc selects the columns per lane.
template <typename R, int RECON, int RS, int NV>
cudaError_t launch_march_one(const StageParams& p, dim3 grid, cudaStream_t s) {
  const int ntiles = (int)grid.x;
  const dim3 blocks((ntiles + kMarchWarps - 1) / kMarchWarps), threads(kMarchWarps * 32);
  if constexpr (sizeof(R) == 4) {
    if (p.nc == 1) return launch_march_nc<R, RECON, RS, NV, 1>(p, blocks, threads, ntiles, s);
    if (p.nc == 3) return launch_march_nc<R, RECON, RS, NV, 3>(p, blocks, threads, ntiles, s);
  }
  if (p.nc != 2) return cudaErrorInvalidValue;
  return launch_march_nc<R, RECON, RS, NV, 2>(p, blocks, threads, ntiles, s);
}

}  // namespace jx

namespace jx {

// Entry points for one (reconstruction, Riemann solver): each march_*.cu
// translation unit instantiates one pair, so the build compiles the kernels
// in parallel.
template <int RECON, int RS>
cudaError_t launch_march_rs(int dtype, const StageParams& p, dim3 grid, cudaStream_t s) {
  const bool three = p.nv == 3;
  if (dtype == JX_F64)
    return three ? launch_march_one<double, RECON, RS, 3>(p, grid, s) : launch_march_one<double, RECON, RS, 4>(p, grid, s);
  return three ? launch_march_one<float, RECON, RS, 3>(p, grid, s) : launch_march_one<float, RECON, RS, 4>(p, grid, s);
}

template <typename R, int RECON, int RS, int NV, int NC>
cudaError_t launch_batch_march_k(bool ring, const StageParams* params, const int* offsets, int nsolves, int nwork,
                                 dim3 grid, cudaStream_t s) {
  constexpr int T = kMarchWarps * 32;
  if constexpr (march_ring_on<R, RECON, NC>()) {
    if (ring) {
      march_prefer_shared<stage_kernel_batch_march<R, RECON, RS, NV, NC, true>>();
      stage_kernel_batch_march<R, RECON, RS, NV, NC, true><<<grid, T, march_smem<NC>(), s>>>(params, offsets, nsolves,
                                                                                            nwork);
      return cudaGetLastError();
    }
  }
  stage_kernel_batch_march<R, RECON, RS, NV, NC><<<grid, T, 0, s>>>(params, offsets, nsolves, nwork);
  return cudaGetLastError();
}

template <typename R, int RECON, int RS, int NV>
cudaError_t launch_batch_march_rs_nv(int nc, bool ring, const StageParams* params, const int* offsets, int nsolves,
                                     int nwork, dim3 grid, cudaStream_t s) {
  if constexpr (sizeof(R) == 4) {
    if (nc == 1) return launch_batch_march_k<R, RECON, RS, NV, 1>(ring, params, offsets, nsolves, nwork, grid, s);
    if (nc == 3) return launch_batch_march_k<R, RECON, RS, NV, 3>(ring, params, offsets, nsolves, nwork, grid, s);
  }
  if (nc != 2) return cudaErrorInvalidValue;
  return launch_batch_march_k<R, RECON, RS, NV, 2>(ring, params, offsets, nsolves, nwork, grid, s);
}

// A group's stage in the packed walk where march_packed allows it (the same
// rules as the single-solve launches; batches carry no SGS stress); true if
// launched.
template <int RECON, int RS, int NV, int FORM>
bool launch_batch_march_packed(bool ring, const StageParams* params, const int* offsets, int nsolves, int nwork,
                               dim3 grid, cudaStream_t s) {
  if constexpr (march_packed<float, RECON, RS, NV, 2, FORM>()) {
    if (!ring) {
      if constexpr (march_packed_short<RECON>()) {
        stage_kernel_batch_march_pk<RECON, RS, NV, FORM, false><<<grid, 32, 0, s>>>(params, offsets, nsolves, nwork);
        return true;
      }
    } else if constexpr (march_packed_ring<RECON, RS>()) {
      march_prefer_shared<stage_kernel_batch_march_pk<RECON, RS, NV, FORM, true>>();
      stage_kernel_batch_march_pk<RECON, RS, NV, FORM, true><<<grid, 32, march_smem<2>(), s>>>(params, offsets,
                                                                                              nsolves, nwork);
      return true;
    }
  }
  return false;
}

// Whether a group of (RECON, RS, NV, FORM) at `ring` runs the packed walk.
template <int RECON, int RS, int NV, int FORM>
bool batch_march_packed(bool ring) {
  if constexpr (march_packed<float, RECON, RS, NV, 2, FORM>())
    return ring ? march_packed_ring<RECON, RS>() : march_packed_short<RECON>();
  return false;
}

template <int RECON, int RS>
cudaError_t launch_batch_march_rs(int dtype, int nv, int nc, int ring, int form, const StageParams* params,
                                  const int* offsets, int nsolves, int nwork, dim3 grid, cudaStream_t s) {
  if (dtype == JX_F32 && nc == 2) {
    bool done = false;
    if (nv == 4 && form == kMarchLeanBlend)
      done = launch_batch_march_packed<RECON, RS, 4, kMarchLeanBlend>(ring, params, offsets, nsolves, nwork, grid, s);
    else if (nv == 4 && form == kMarchLeanPlain)
      done = launch_batch_march_packed<RECON, RS, 4, kMarchLeanPlain>(ring, params, offsets, nsolves, nwork, grid, s);
    else if (nv == 3 && form == kMarchGeneric)
      done = launch_batch_march_packed<RECON, RS, 3, kMarchGeneric>(ring, params, offsets, nsolves, nwork, grid, s);
    if (done) return cudaGetLastError();
  }
  if (dtype == JX_F64)
    return nv == 3 ? launch_batch_march_rs_nv<double, RECON, RS, 3>(nc, ring, params, offsets, nsolves, nwork, grid, s)
                   : launch_batch_march_rs_nv<double, RECON, RS, 4>(nc, ring, params, offsets, nsolves, nwork, grid, s);
  return nv == 3 ? launch_batch_march_rs_nv<float, RECON, RS, 3>(nc, ring, params, offsets, nsolves, nwork, grid, s)
                 : launch_batch_march_rs_nv<float, RECON, RS, 4>(nc, ring, params, offsets, nsolves, nwork, grid, s);
}

template <typename Kernel>
int march_occupancy(Kernel kernel, size_t smem = 0) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kMarchWarps * 32, smem) != cudaSuccess) return 0;
  return n;
}

// Resident marching blocks per SM (single-solve or batch kernel).
// Resident blocks per SM of the kernel a launch would run: the batch
// kernel, or the single-solve kernel in its lean blend form (float32, two or
// three columns per lane, an inviscid problem without drag) or its generic
// form, with the ring's shared memory where the ring is built.
template <typename R, int RECON, int RS, int NV, int NC, int FORM>
int march_single_occupancy() {
  if constexpr (march_packed<R, RECON, RS, NV, NC, FORM>() && march_packed_ring<RECON, RS>()) {
    if constexpr (RECON == JX_PPM4) {
      march_prefer_shared<stage_kernel_march_pk_x<RS, NV, FORM>>();
      return march_occupancy(stage_kernel_march_pk_x<RS, NV, FORM>, march_smem<2>());
    } else {
      march_prefer_shared<stage_kernel_march_pk<RECON, RS, NV, FORM, true>>();
      return march_occupancy(stage_kernel_march_pk<RECON, RS, NV, FORM, true>, march_smem<2>());
    }
  }
  constexpr bool ring = march_ring_on<R, RECON, NC>();
  if constexpr (ring) {
    march_prefer_shared<stage_kernel_march<R, RECON, RS, NV, NC, FORM, true>>();
    return march_occupancy(stage_kernel_march<R, RECON, RS, NV, NC, FORM, true>, march_smem<NC>());
  }
  return march_occupancy(stage_kernel_march<R, RECON, RS, NV, NC, FORM>);
}

// Resident blocks of the batched packed kernel of FORM, or 0 where the
// packed walk does not run.
template <typename R, int RECON, int RS, int NV, int NC, int FORM>
int batch_packed_occupancy(bool ring) {
  if constexpr (sizeof(R) == 4 && NC == 2 && march_packed<R, RECON, RS, NV, NC, FORM>()) {
    if (ring) {
      if constexpr (march_packed_ring<RECON, RS>()) {
        march_prefer_shared<stage_kernel_batch_march_pk<RECON, RS, NV, FORM, true>>();
        return march_occupancy(stage_kernel_batch_march_pk<RECON, RS, NV, FORM, true>, march_smem<2>());
      }
    } else if constexpr (march_packed_short<RECON>()) {
      return march_occupancy(stage_kernel_batch_march_pk<RECON, RS, NV, FORM, false>);
    }
  }
  return 0;
}

template <typename R, int RECON, int RS, int NV, int NC>
int march_blocks_per_sm_nv(int kind) {
  if (kind == kMarchBatchPacked || kind == kMarchBatchPackedRing) {
    const int n = batch_packed_occupancy<R, RECON, RS, NV, NC, kMarchLeanBlend>(kind == kMarchBatchPackedRing);
    if (n > 0) return n;
    kind = kind == kMarchBatchPackedRing ? kMarchBatchRing : kMarchBatch;
  }
  if (kind == kMarchBatch || kind == kMarchBatchRing) {
    // Generic groups of 3-variable solves run the packed walk where it is used.
    const int n = batch_packed_occupancy<R, RECON, RS, NV, NC, kMarchGeneric>(kind == kMarchBatchRing);
    if (n > 0) return n;
  }
  if (kind == kMarchBatch || kind == kMarchBatchRing) {
    if constexpr (march_ring_on<R, RECON, NC>()) {
      if (kind == kMarchBatchRing) {
        march_prefer_shared<stage_kernel_batch_march<R, RECON, RS, NV, NC, true>>();
        return march_occupancy(stage_kernel_batch_march<R, RECON, RS, NV, NC, true>, march_smem<NC>());
      }
    }
    return march_occupancy(stage_kernel_batch_march<R, RECON, RS, NV, NC>);
  }
  if constexpr (sizeof(R) == 4 && NC > 1)
    if (kind == kMarchSingleLean) return march_single_occupancy<R, RECON, RS, NV, NC, kMarchLeanBlend>();
  return march_single_occupancy<R, RECON, RS, NV, NC, kMarchGeneric>();
}

template <typename R, int RECON, int RS, int NC>
int march_blocks_per_sm_nc(int nv, int kind) {
  return nv == 3 ? march_blocks_per_sm_nv<R, RECON, RS, 3, NC>(kind) : march_blocks_per_sm_nv<R, RECON, RS, 4, NC>(kind);
}

template <typename R, int RECON, int RS>
int march_blocks_per_sm_rs(int nv, int nc, int kind) {
  if constexpr (sizeof(R) == 4) {
    if (nc == 1) return march_blocks_per_sm_nc<R, RECON, RS, 1>(nv, kind);
    if (nc == 3) return march_blocks_per_sm_nc<R, RECON, RS, 3>(nv, kind);
  }
  return nc == 2 ? march_blocks_per_sm_nc<R, RECON, RS, 2>(nv, kind) : 0;
}

template <int RECON, int RS>
int march_blocks_per_sm_rs_dtype(int dtype, int nv, int nc, int kind) {
  if ((kind == kMarchBatchPacked || kind == kMarchBatchPackedRing) &&
      !(dtype == JX_F32 && nv == 4 && nc == 2 &&
        batch_march_packed<RECON, RS, 4, kMarchLeanBlend>(kind == kMarchBatchPackedRing)))
    kind = kind == kMarchBatchPackedRing ? kMarchBatchRing : kMarchBatch;
  return dtype == JX_F64 ? march_blocks_per_sm_rs<double, RECON, RS>(nv, nc, kind)
                         : march_blocks_per_sm_rs<float, RECON, RS>(nv, nc, kind);
}

}  // namespace jx
