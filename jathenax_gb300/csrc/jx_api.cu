// C ABI (include/jx.h): argument checks, workspace layout, and the launch
// sequences of one RK stage, one full step and the forcing passes.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "jx_aux.cuh"
#include "jx_internal.h"

using namespace jx;

namespace {

thread_local char g_error[512] = "";

jx_status fail(jx_status code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
  return code;
}

jx_status cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) return fail(JX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return JX_OK;
}

// hydro.py:20-36 (AthenaK driver.cpp): (gamma0, gamma1, beta, delta or NaN).
struct RkRow {
  double g0, g1, beta, delta;
  bool has_delta;
};
const RkRow kRk2[2] = {{0.0, 1.0, 1.0, 0.0, false}, {0.5, 0.5, 0.5, 0.0, false}};
const RkRow kRk3[3] = {{0.0, 1.0, 1.0, 0.0, false},
                       {0.25, 0.75, 0.25, 0.0, false},
                       {2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0, 0.0, false}};
const RkRow kRk4[4] = {
    {0.0, 1.0, 1.193743905974738, 0.0, false},
    {0.121098479554482, 0.721781678111411, 0.099279895495783, 0.217683334308543, true},
    {-3.843833699660025, 2.121209265338722, 1.131678018054042, 1.065841341361089, true},
    {0.546370891121863, 0.198653035682705, 0.310665766509336, 0.0, true}};

const RkRow* rk_rows(int integrator) {
  return integrator == JX_RK2 ? kRk2 : (integrator == JX_RK3 ? kRk3 : kRk4);
}

constexpr size_t kSmemLimit = 227 * 1024;
constexpr size_t kSmemDefaultCap = 112 * 1024;  // keep two CTAs per SM by default

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

bool finite_nonneg(double x) { return isfinite(x) && x >= 0.0; }

jx_status check_desc(const jx_desc* d) {
  if (!d) return fail(JX_ERR_INVALID, "null descriptor");
  if (d->ny < 1 || d->nx < 1) return fail(JX_ERR_INVALID, "grid must have at least one cell per axis");
  if (d->nvar < 3 || d->nvar > 64) return fail(JX_ERR_INVALID, "nvar must be in [3, 64]");
  if ((int64_t)d->ny * d->nx > ((int64_t)1 << 31) - 1)
    return fail(JX_ERR_INVALID, "grid larger than 2^31 cells");
  if (d->dtype != JX_F64 && d->dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", d->dtype);
  if (d->recon < JX_DC || d->recon > JX_WENOZ) return fail(JX_ERR_UNSUPPORTED, "unknown reconstruction %d", d->recon);
  if (d->rsolver < JX_LLF || d->rsolver > JX_ROE) return fail(JX_ERR_UNSUPPORTED, "unknown Riemann solver %d", d->rsolver);
  if (d->integrator < JX_RK2 || d->integrator > JX_RK4)
    return fail(JX_ERR_UNSUPPORTED, "unknown integrator %d", d->integrator);
  if (!(isfinite(d->dx) && d->dx > 0 && isfinite(d->dy) && d->dy > 0))
    return fail(JX_ERR_INVALID, "dx and dy must be finite and positive");
  if (!(isfinite(d->cs) && d->cs > 0)) return fail(JX_ERR_INVALID, "cs must be finite and positive");
  if (!isfinite(d->dfloor)) return fail(JX_ERR_INVALID, "dfloor must be finite");
  if (!finite_nonneg(d->viscosity)) return fail(JX_ERR_INVALID, "viscosity must be finite and nonnegative");
  if (!finite_nonneg(d->smagorinsky_cs)) return fail(JX_ERR_INVALID, "smagorinsky_cs must be finite and nonnegative");
  if (!finite_nonneg(d->drag_rate)) return fail(JX_ERR_INVALID, "drag_rate must be finite and nonnegative");
  if (d->tile_x < 0 || d->tile_y < 0 || d->tile_x > 256 || d->tile_y > 256)
    return fail(JX_ERR_INVALID, "tile_x/tile_y must be in [0, 256]");
  return JX_OK;
}

struct Tile {
  int tx, ty, tiles_x, tiles_y;
  size_t smem;       // generic kernel
  bool fast_shape;   // 3/4 variables at tile width 32: the fast kernel applies
  size_t fast_smem;  // fast kernel
  // Register-marching kernel (3/4 variables): march_tile_x(mnc) x mty tiles,
  // mnc columns per lane. The shared-memory tile above stays resolved for
  // stages that fall back (trace outputs requested, 4-variable arrays not
  // 16-byte aligned).
  bool march;
  int mnc, mty, mtiles_x, mtiles_y;
  size_t cfl_slots;  // CFL partial slots the workspace holds
};

int sm_count();

// Resident marching blocks per SM for this descriptor on the current device
// (cached; 4 when the device cannot be queried).
// Resident marching blocks per SM for a descriptor's solve: the kernel its
// stages run (the lean form for an inviscid problem without drag, whose
// register count, and so occupancy, can differ from the generic form's).
int march_occupancy(const jx_desc* d, int nc) {
  static int cache[64][2][5][3][2][3][2];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 4;
  const bool lean = d->viscosity == 0.0 && d->smagorinsky_cs == 0.0 && d->drag_rate == 0.0;
  int& c = cache[dev][d->dtype][d->recon][d->rsolver][d->nvar - 3][nc - 1][lean];
  if (c == 0) {
    int n = 0;
    switch (d->recon) {
      case JX_DC: n = march_blocks_per_sm_dc(d->dtype, d->rsolver, d->nvar, nc, lean ? kMarchSingleLean : kMarchSingle); break;
      case JX_PLM: n = march_blocks_per_sm_plm(d->dtype, d->rsolver, d->nvar, nc, lean ? kMarchSingleLean : kMarchSingle); break;
      case JX_PPM4: n = march_blocks_per_sm_ppm4(d->dtype, d->rsolver, d->nvar, nc, lean ? kMarchSingleLean : kMarchSingle); break;
      case JX_PPMX: n = march_blocks_per_sm_ppmx(d->dtype, d->rsolver, d->nvar, nc, lean ? kMarchSingleLean : kMarchSingle); break;
      default: n = march_blocks_per_sm_wenoz(d->dtype, d->rsolver, d->nvar, nc, lean ? kMarchSingleLean : kMarchSingle); break;
    }
    if (n < 1) {
      cudaGetLastError();
      return 4;
    }
    c = n;
  }
  return c;
}

// Rows of an automatic marching tile: the height whose tiles, spread over
// the resident warp slots of the device, finish soonest. A tile of h rows
// costs about h + 2.5 row-updates (the 6 leading rows of the walk do the y
// work only); the grid runs in ceil(tiles / slots) rounds. Besides a fixed
// list the candidates include the shortest height whose tiles all fit in one
// round (every warp walks one tall tile; e.g. 121 rows at 4096^2 with 16
// resident warps per SM: 2414 tiles on 2432 slots).
int march_rows(const jx_desc* d, int nc) {
  static const int kRows[] = {8, 12, 16, 24, 32, 48, 64};
  const int64_t slots = (int64_t)sm_count() * march_occupancy(d, nc) * kMarchWarps;
  const int64_t cols = (d->nx + march_tile_x(nc) - 1) / march_tile_x(nc);
  int cand[8];
  int ncand = 0;
  for (int h : kRows) cand[ncand++] = h;
  const int64_t rows_per_round = slots / cols;  // tile rows that fit in one round
  if (rows_per_round >= 1) {
    const int64_t h1 = (d->ny + rows_per_round - 1) / rows_per_round;
    if (h1 > kRows[6] && h1 <= d->ny) cand[ncand++] = (int)h1;
  }
  int best = kRows[0];
  double best_cost = 1e300;
  for (int i = 0; i < ncand; ++i) {
    const int h = cand[i];
    const int64_t tiles = cols * ((d->ny + h - 1) / h);
    const int64_t rounds = (tiles + slots - 1) / slots;
    const double cost = (double)rounds * (h + 2.5);
    if (cost <= best_cost) {
      best_cost = cost;
      best = h;
    }
  }
  return best;
}

jx_status resolve_tile(const jx_desc* d, Tile* t, bool device = true) {
  // Automatic tiles: float32 marches with two columns per lane (WENO-Z,
  // whose long stencil needs the registers, with one: 1.36 against 1.48 ms
  // per 4096² stage at the best heights); float64, bound by the FP64 pipe,
  // keeps the shared-memory tile, which evaluates no halo faces twice. An
  // explicit tile width of 26, 58 or 90 asks for the marching kernel with
  // 1, 2 or 3 columns per lane (float64: 58 only).
  const bool three_four = d->nvar == 3 || d->nvar == 4;
  const int want_nc = march_cols(d->tile_x);
  const bool march = three_four && (want_nc > 0 || (d->tile_x == 0 && d->tile_y == 0 && d->dtype == JX_F32));
  const int nc = want_nc > 0 ? want_nc : (d->dtype == JX_F32 && d->recon == JX_WENOZ ? 1 : 2);
  if (march && d->dtype == JX_F64 && nc != 2)
    return fail(JX_ERR_INVALID, "float64 marching tiles are %d columns wide, not %d", kMarchTileX, d->tile_x);
  int tx = d->tile_x > 0 && !march ? d->tile_x : 32;
  int ty = d->tile_y > 0 && !march ? d->tile_y : 16;
  size_t smem = stage_smem_bytes(d->recon, d->dtype, d->nvar, tx, ty);
  if (march || (d->tile_x == 0 && d->tile_y == 0)) {
    while (smem > kSmemDefaultCap && ty > 4) {
      ty /= 2;
      smem = stage_smem_bytes(d->recon, d->dtype, d->nvar, tx, ty);
    }
    while (smem > kSmemDefaultCap && tx > 8) {
      tx /= 2;
      smem = stage_smem_bytes(d->recon, d->dtype, d->nvar, tx, ty);
    }
  }
  if (smem > kSmemLimit)
    return fail(JX_ERR_INVALID, "tile %dx%d needs %zu bytes of shared memory (limit %zu)", tx, ty, smem, kSmemLimit);
  t->fast_shape = three_four && tx == 32;
  t->fast_smem = t->fast_shape ? fast_smem_bytes(d->recon, d->dtype, ty) : 0;
  if (t->fast_smem > kSmemLimit)
    return fail(JX_ERR_INVALID, "tile 32x%d needs %zu bytes of shared memory (limit %zu)", ty, t->fast_smem,
                kSmemLimit);
  t->tx = tx;
  t->ty = ty;
  t->tiles_x = (d->nx + tx - 1) / tx;
  t->tiles_y = (d->ny + ty - 1) / ty;
  t->smem = smem;
  if ((int64_t)t->tiles_x * t->tiles_y > ((int64_t)1 << 31) - 1) return fail(JX_ERR_INVALID, "too many tiles");
  t->march = march;
  t->mnc = t->mty = t->mtiles_x = t->mtiles_y = 0;
  size_t slots = (size_t)t->tiles_x * t->tiles_y;
  if (march) {
    if (d->tile_y > 0 && d->tile_y < kMarchMinRows)
      return fail(JX_ERR_INVALID, "marching tiles need at least %d rows", kMarchMinRows);
    // The workspace covers the shortest automatic marching tile, so its
    // size does not depend on the device.
    const int64_t cols = (d->nx + march_tile_x(nc) - 1) / march_tile_x(nc);
    const int rows_min = d->tile_y > 0 ? d->tile_y : kMarchMinRows;
    const size_t mslots = (size_t)(cols * ((d->ny + rows_min - 1) / rows_min));
    if (mslots > slots) slots = mslots;
    t->mnc = nc;
    t->mty = d->tile_y > 0 ? d->tile_y : (device ? march_rows(d, nc) : kMarchMinRows);
    t->mtiles_x = (int)cols;
    t->mtiles_y = (d->ny + t->mty - 1) / t->mty;
  }
  t->cfl_slots = slots;
  return JX_OK;
}

struct Layout {
  size_t scal, cfl, p1, box, total;
};

Layout layout_for(const jx_desc* d, const Tile& t) {
  Layout L;
  size_t off = kWsHeader;
  L.scal = off;
  off += 256;
  L.cfl = off;
  size_t slots = t.cfl_slots;
  if (slots < (size_t)kCflBlocksMax) slots = kCflBlocksMax;
  off = align256(off + slots * kCflSlots * sizeof(double));
  L.p1 = off;  // forcing moments, 8 per block
  off = align256(off + (size_t)kForceBlocksMax * 8 * sizeof(double));
  L.box = off;
  off = align256(off + (size_t)kForceBlocksMax * d->nvar * sizeof(double));
  L.total = off;
  return L;
}

struct Ws {
  WsHeader* header;
  double *scal, *cfl, *p1, *box;
};

jx_status bind_ws(const jx_desc* d, const Tile& t, void* ws, size_t bytes, Ws* w) {
  if (!ws) return fail(JX_ERR_WORKSPACE, "null workspace");
  if (((uintptr_t)ws & 255) != 0) return fail(JX_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  Layout L = layout_for(d, t);
  if (bytes < L.total) return fail(JX_ERR_WORKSPACE, "workspace has %zu bytes, needs %zu", bytes, L.total);
  char* b = static_cast<char*>(ws);
  w->header = reinterpret_cast<WsHeader*>(b);
  w->scal = reinterpret_cast<double*>(b + L.scal);
  w->cfl = reinterpret_cast<double*>(b + L.cfl);
  w->p1 = reinterpret_cast<double*>(b + L.p1);
  w->box = reinterpret_cast<double*>(b + L.box);
  return JX_OK;
}

DtParams dt_params(const jx_desc* d) {
  DtParams q;
  q.dx = d->dx;
  q.dy = d->dy;
  q.nu = d->viscosity;
  q.smag_cs = d->smagorinsky_cs;
  q.smag_c = d->smagorinsky_cs * d->smagorinsky_cs * d->dx * d->dy;
  q.drag = d->drag_rate;
  return q;
}

CflParams cfl_params(const jx_desc* d, const void* X, const jx_clock* clock, const Ws& w) {
  CflParams q;
  q.X = X;
  q.clock = clock;
  q.partials = w.cfl;
  q.header = w.header;
  q.ny = d->ny;
  q.nx = d->nx;
  q.nv = d->nvar;
  q.smag = d->smagorinsky_cs > 0.0;
  q.cs = d->cs;
  q.dfloor = d->dfloor;
  q.inv_dx = 1.0 / d->dx;
  q.inv_dy = 1.0 / d->dy;
  q.inv_4dx = 1.0 / (4.0 * d->dx);
  q.inv_4dy = 1.0 / (4.0 * d->dy);
  return q;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

// The marching kernel applies unless trace outputs are requested (it writes
// none) or a 4-variable array is not 16-byte aligned (128-bit accesses).
bool use_march(const jx_desc* d, const StageParams& p, const Tile& t) {
  return t.march && !p.trace_on &&
         (d->nvar == 3 ||
          (aligned16(p.U) && aligned16(p.V) && aligned16(p.Uout) && (p.Vout == nullptr || aligned16(p.Vout))));
}

cudaError_t launch_march(int recon, int dtype, int rsolver, const StageParams& p, dim3 grid, cudaStream_t s) {
  switch (recon) {
    case JX_DC: return launch_march_dc(dtype, rsolver, p, grid, s);
    case JX_PLM: return launch_march_plm(dtype, rsolver, p, grid, s);
    case JX_PPM4: return launch_march_ppm4(dtype, rsolver, p, grid, s);
    case JX_PPMX: return launch_march_ppmx(dtype, rsolver, p, grid, s);
    default: return launch_march_wenoz(dtype, rsolver, p, grid, s);
  }
}

cudaError_t launch_stage(const jx_desc* d, const StageParams& p, const Tile& t, cudaStream_t s) {
  if (use_march(d, p, t)) {
    StageParams m = p;
    m.tx = march_tile_x(t.mnc);
    m.nc = t.mnc;
    m.ty = t.mty;
    m.tiles_x = t.mtiles_x;
    return launch_march(d->recon, d->dtype, d->rsolver, m, dim3((unsigned)((int64_t)t.mtiles_x * t.mtiles_y)), s);
  }
  dim3 grid((unsigned)((int64_t)t.tiles_x * t.tiles_y));
  // The fast kernel reads/writes 4-variable cells with 128-bit accesses.
  const bool fast = t.fast_shape && (d->nvar == 3 || (aligned16(p.U) && aligned16(p.V) && aligned16(p.Uout) &&
                                                      (p.Vout == nullptr || aligned16(p.Vout))));
  if (fast) {
    switch (d->recon) {
      case JX_DC: return launch_fast_dc(d->dtype, d->rsolver, p, grid, t.fast_smem, s);
      case JX_PLM: return launch_fast_plm(d->dtype, d->rsolver, p, grid, t.fast_smem, s);
      case JX_PPM4: return launch_fast_ppm4(d->dtype, d->rsolver, p, grid, t.fast_smem, s);
      case JX_PPMX: return launch_fast_ppmx(d->dtype, d->rsolver, p, grid, t.fast_smem, s);
      default: return launch_fast_wenoz(d->dtype, d->rsolver, p, grid, t.fast_smem, s);
    }
  }
  switch (d->recon) {
    case JX_DC: return launch_stage_dc(d->dtype, d->rsolver, p, grid, t.smem, s);
    case JX_PLM: return launch_stage_plm(d->dtype, d->rsolver, p, grid, t.smem, s);
    case JX_PPM4: return launch_stage_ppm4(d->dtype, d->rsolver, p, grid, t.smem, s);
    case JX_PPMX: return launch_stage_ppmx(d->dtype, d->rsolver, p, grid, t.smem, s);
    default: return launch_stage_wenoz(d->dtype, d->rsolver, p, grid, t.smem, s);
  }
}

// Launch parameters of one stage (hydro.py:101-143); validated by the caller.
StageParams make_stage_params(const jx_desc* d, const Tile& t, const Ws& w, int stage, const void* U_in,
                              const void* V_in, void* U_out, void* V_out, const void* tau, int force_follows,
                              jx_clock* clock, const jx_trace* trace) {
  const int n = jx_num_stages(d->integrator);
  const RkRow& row = rk_rows(d->integrator)[stage - 1];
  const bool last = stage == n;
  StageParams p;
  memset(&p, 0, sizeof(p));
  p.U = U_in;
  p.V = V_in;
  p.Uout = U_out;
  p.Vout = row.has_delta ? V_out : nullptr;
  p.tau = tau;
  p.clock = clock;
  p.partials = w.cfl;
  p.header = w.header;
  if (trace) p.trace = *trace;
  p.trace_on = trace != nullptr;
  p.ny = d->ny;
  p.nx = d->nx;
  p.nv = d->nvar;
  p.tx = t.tx;
  p.ty = t.ty;
  p.tiles_x = t.tiles_x;
  p.dx = d->dx;
  p.dy = d->dy;
  p.inv_dx = 1.0 / d->dx;
  p.inv_dy = 1.0 / d->dy;
  p.inv_4dx = 1.0 / (4.0 * d->dx);
  p.inv_4dy = 1.0 / (4.0 * d->dy);
  p.cs = d->cs;
  p.dfloor = d->dfloor;
  p.nu = d->viscosity;
  p.smag_c = d->smagorinsky_cs * d->smagorinsky_cs * d->dx * d->dy;
  p.drag = d->drag_rate;
  p.g0 = row.g0;
  p.g1 = row.g1;
  p.beta = row.beta;
  p.delta = row.delta;
  p.has_delta = row.has_delta;
  p.blend = row.g0 != 0.0 && row.g0 + row.g1 == 1.0;  // hydro.py:46
  p.floor_v = !(d->integrator == JX_RK4 && stage >= 3);  // V is still the floored step-start state
  p.floor_out = !(last && force_follows);
  p.want_cfl = last && !force_follows && !(d->smagorinsky_cs > 0.0);
  p.visc_on = d->viscosity > 0.0 || d->smagorinsky_cs > 0.0;
  p.smag_on = d->smagorinsky_cs > 0.0;
  p.drag_on = d->drag_rate > 0.0;
  fill_stage_consts(p.cd, p);
  fill_stage_consts(p.cf, p);
  return p;
}

jx_status do_stage(const jx_desc* d, const Tile& t, const Ws& w, int stage, const void* U_in,
                   const void* V_in, void* U_out, void* V_out, const void* tau, int force_follows,
                   jx_clock* clock, const jx_trace* trace, cudaStream_t s) {
  const int n = jx_num_stages(d->integrator);
  if (stage < 1 || stage > n) return fail(JX_ERR_INVALID, "stage %d outside 1..%d", stage, n);
  if (!U_in || !V_in || !U_out || !clock) return fail(JX_ERR_INVALID, "null state or clock pointer");
  const RkRow& row = rk_rows(d->integrator)[stage - 1];
  if (U_in == U_out || (row.has_delta && U_in == V_out))
    return fail(JX_ERR_INVALID, "U_in must not alias an output");
  const StageParams p =
      make_stage_params(d, t, w, stage, U_in, V_in, U_out, V_out, tau, force_follows, clock, trace);
  return cuda_check(launch_stage(d, p, t, s), "stage kernel");
}

ForceParams force_params(const jx_desc* d, const jx_forcing* f, void* U, jx_clock* clock, const jx_trace* trace,
                         const Ws& w) {
  ForceParams q;
  memset(&q, 0, sizeof(q));
  q.clock = clock;
  q.U = U;
  q.Uw = U;
  q.raw = f->raw_force;
  q.p1 = w.p1;
  q.scal = w.scal;
  q.partials = w.cfl;
  q.header = w.header;
  if (trace) {
    q.before_kick = trace->before_kick;
    q.acceleration = trace->acceleration;
    q.conserved = trace->conserved;
  }
  q.ny = d->ny;
  q.nx = d->nx;
  q.nv = d->nvar;
  force_decomposition((int64_t)d->ny * d->nx, &q.nblk, &q.chunk);
  q.want_cfl = !(d->smagorinsky_cs > 0.0);
  q.dfloor = d->dfloor;
  q.cs = d->cs;
  return q;
}

RenderParams render_params(const jx_desc* d, const jx_forcing* f, jx_clock* clock) {
  RenderParams q;
  memset(&q, 0, sizeof(q));
  q.clock = clock;
  q.table = f->table;
  q.cos_x = f->cos_x;
  q.sin_x = f->sin_x;
  q.cos_y = f->cos_y;
  q.sin_y = f->sin_y;
  q.raw = f->raw_force;
  q.ny = d->ny;
  q.nx = d->nx;
  q.n_modes = f->n_modes;
  q.n_updates = f->n_updates;
  return q;
}

jx_status do_kick(const jx_desc* d, const jx_forcing* f, void* U, jx_clock* clock,
                  const jx_trace* trace, const Ws& w, cudaStream_t s) {
  if (!f || !f->raw_force) return fail(JX_ERR_INVALID, "forcing needs a raw_force buffer");
  if (!U || !clock) return fail(JX_ERR_INVALID, "null state or clock pointer");
  return cuda_check(launch_force_kick(d->dtype, force_params(d, f, U, clock, trace, w), s), "force kick kernels");
}

}  // namespace

extern "C" {

const char* jx_last_error(void) { return g_error; }

const char* jx_version(void) { return "jx 0.1.0 (sm_103a)"; }

int32_t jx_num_stages(int32_t integrator) {
  return integrator == JX_RK2 ? 2 : (integrator == JX_RK3 ? 3 : (integrator == JX_RK4 ? 4 : 0));
}

jx_status jx_check_desc(const jx_desc* d) { return check_desc(d); }

jx_status jx_tile_info(const jx_desc* d, int32_t* tile_x, int32_t* tile_y, int64_t* smem_bytes) {
  jx_status st = check_desc(d);
  if (st) return st;
  Tile t;
  if ((st = resolve_tile(d, &t))) return st;
  if (tile_x) *tile_x = t.march ? march_tile_x(t.mnc) : t.tx;
  if (tile_y) *tile_y = t.march ? t.mty : t.ty;
  if (smem_bytes) *smem_bytes = t.march ? 0 : (int64_t)t.smem;
  return JX_OK;
}

jx_status jx_workspace_bytes(const jx_desc* d, size_t* bytes) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!bytes) return fail(JX_ERR_INVALID, "null output pointer");
  Tile t;
  if ((st = resolve_tile(d, &t, false))) return st;
  *bytes = layout_for(d, t).total;
  return JX_OK;
}

jx_status jx_recover(const jx_desc* d, const void* U, void* U_out, void* W, jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!U) return fail(JX_ERR_INVALID, "null state pointer");
  return cuda_check(launch_recover(d->dtype, U, U_out, W, (int64_t)d->ny * d->nx, d->nvar, d->dfloor,
                                   (cudaStream_t)s),
                    "recover kernel");
}

jx_status jx_timestep(const jx_desc* d, const void* W, double cfl, double prev_dt, double time,
                      double tlim, double* dt_out, void* workspace, size_t workspace_bytes,
                      jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!W || !dt_out) return fail(JX_ERR_INVALID, "null W or dt_out");
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  CflParams q = cfl_params(d, W, nullptr, w);
  if ((st = cuda_check(launch_cfl(d->dtype, true, q, (cudaStream_t)s), "cfl kernel"))) return st;
  return cuda_check(launch_timestep_finish(dt_params(d), w.cfl, w.header, prev_dt, time, tlim, cfl,
                                           dt_out, (cudaStream_t)s),
                    "timestep finisher");
}

jx_status jx_stage(const jx_desc* d, int32_t stage, const void* U_in, const void* V_in, void* U_out,
                   void* V_out, const void* tau, int32_t force_follows, jx_clock* clock,
                   const jx_trace* trace, void* workspace, size_t workspace_bytes, jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  return do_stage(d, t, w, stage, U_in, V_in, U_out, V_out, tau, force_follows, clock, trace,
                  (cudaStream_t)s);
}

jx_status jx_cfl_partials(const jx_desc* d, const void* U, void* workspace, size_t workspace_bytes,
                          jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!U) return fail(JX_ERR_INVALID, "null state pointer");
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  CflParams q = cfl_params(d, U, nullptr, w);
  return cuda_check(launch_cfl(d->dtype, false, q, (cudaStream_t)s), "cfl kernel");
}

jx_status jx_begin_step(const jx_desc* d, jx_clock* clock, int32_t forced, void* workspace,
                        size_t workspace_bytes, jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!clock) return fail(JX_ERR_INVALID, "null clock");
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  return cuda_check(launch_begin_step(dt_params(d), clock, w.cfl, w.header, forced, (cudaStream_t)s),
                    "begin-step kernel");
}

jx_status jx_force_render(const jx_desc* d, const jx_forcing* f, jx_clock* clock, jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!f || !clock || !f->table || !f->cos_x || !f->sin_x || !f->cos_y || !f->sin_y || !f->raw_force)
    return fail(JX_ERR_INVALID, "incomplete forcing tables");
  if (f->n_modes < 1 || f->n_updates < 1) return fail(JX_ERR_INVALID, "forcing needs modes and updates");
  return cuda_check(launch_render(d->dtype, render_params(d, f, clock), (cudaStream_t)s), "render kernel");
}

jx_status jx_force_kick(const jx_desc* d, const jx_forcing* f, void* U, jx_clock* clock,
                        const jx_trace* trace, void* workspace, size_t workspace_bytes, jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  return do_kick(d, f, U, clock, trace, w, (cudaStream_t)s);
}

jx_status jx_step(const jx_desc* d, void* S, void* A, void* B, const jx_forcing* forcing,
                  jx_clock* clock, void* workspace, size_t workspace_bytes, jx_stream stream) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!S || !A || !B || !clock) return fail(JX_ERR_INVALID, "null state, scratch or clock pointer");
  if (S == A || S == B || A == B) return fail(JX_ERR_INVALID, "S, A and B must be distinct buffers");
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int forced = forcing != nullptr;
  if ((st = cuda_check(launch_begin_step(dt_params(d), clock, w.cfl, w.header, forced, s), "begin-step kernel")))
    return st;
  if (forced && (st = jx_force_render(d, forcing, clock, stream))) return st;
  const int n = jx_num_stages(d->integrator);
  // S -> A -> B -> A ... -> S; the saved register stays in S (pointwise).
  const void* in = S;
  for (int stage = 1; stage <= n; ++stage) {
    void* out = stage == n ? S : (stage % 2 == 1 ? A : B);
    if ((st = do_stage(d, t, w, stage, in, S, out, stage == n ? nullptr : S, nullptr, forced, clock,
                       nullptr, s)))
      return st;
    in = out;
  }
  if (forced && (st = do_kick(d, forcing, S, clock, nullptr, w, s))) return st;
  if (d->smagorinsky_cs > 0.0) {
    CflParams q = cfl_params(d, S, clock, w);
    if ((st = cuda_check(launch_cfl(d->dtype, false, q, s), "cfl kernel"))) return st;
  }
  return JX_OK;
}

jx_status jx_rk_stage(int32_t dtype, int64_t n, const void* U, const void* V, const void* div, double dt,
                      double gam0, double gam1, double beta, double delta, int32_t has_delta,
                      void* U_out, void* V_out, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (n < 0 || (n > 0 && (!U || !V || !div || !U_out))) return fail(JX_ERR_INVALID, "bad rk_stage arguments");
  const int blend = gam0 != 0.0 && gam0 + gam1 == 1.0;
  return cuda_check(launch_rk_stage(dtype, n, U, V, div, U_out, V_out, dt, gam0, gam1, beta, delta, has_delta,
                                    blend, (cudaStream_t)s),
                    "rk_stage kernel");
}

jx_status jx_flux_divergence(int32_t dtype, int32_t ny, int32_t nx, int32_t nv, const void* flux_x,
                             const void* flux_y, double dx, double dy, void* div, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (ny < 0 || nx < 0 || nv < 1) return fail(JX_ERR_INVALID, "bad shape");
  if ((int64_t)ny * nx * nv > 0 && (!flux_x || !flux_y || !div)) return fail(JX_ERR_INVALID, "null array");
  return cuda_check(launch_divergence(dtype, ny, nx, nv, flux_x, flux_y, 1.0 / dx, 1.0 / dy, div, (cudaStream_t)s),
                    "divergence kernel");
}

jx_status jx_stress_face_fluxes(int32_t dtype, int32_t ny, int32_t nx, const void* tau, void* flux_x,
                                void* flux_y, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (ny < 0 || nx < 0) return fail(JX_ERR_INVALID, "bad shape");
  if ((int64_t)ny * nx > 0 && (!tau || !flux_x || !flux_y)) return fail(JX_ERR_INVALID, "null array");
  return cuda_check(launch_stress_faces(dtype, ny, nx, tau, flux_x, flux_y, (cudaStream_t)s), "stress kernel");
}

jx_status jx_box_sums(const jx_desc* d, const void* U, double* out, void* workspace, size_t workspace_bytes,
                      jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!U || !out) return fail(JX_ERR_INVALID, "null pointer");
  Tile t;
  Ws w;
  if ((st = resolve_tile(d, &t)) || (st = bind_ws(d, t, workspace, workspace_bytes, &w))) return st;
  return cuda_check(launch_box_sums(d->dtype, U, (int64_t)d->ny * d->nx, d->nvar, w.box, out, (cudaStream_t)s),
                    "box-sum kernels");
}

jx_status jx_face_states(int32_t dtype, int32_t recon, int32_t ny, int32_t nx, int32_t nv, const void* W,
                         int32_t axis, double dfloor, void* left, void* right, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (recon < JX_DC || recon > JX_WENOZ) return fail(JX_ERR_UNSUPPORTED, "unknown reconstruction %d", recon);
  if (axis != 0 && axis != 1) return fail(JX_ERR_INVALID, "axis must be 0 (y) or 1 (x)");
  if (ny < 0 || nx < 0 || nv < 1) return fail(JX_ERR_INVALID, "bad shape");
  if ((int64_t)ny * nx * nv > 0 && (!W || !left || !right)) return fail(JX_ERR_INVALID, "null array");
  static const FaceStatesLauncher table[5] = {face_states_dc, face_states_plm, face_states_ppm4, face_states_ppmx,
                                              face_states_wenoz};
  return cuda_check(table[recon](dtype, W, ny, nx, nv, axis, dfloor, left, right, (cudaStream_t)s),
                    "face-state kernel");
}

jx_status jx_face_flux(int32_t dtype, int32_t rsolver, int64_t nface, int32_t nv, int32_t axis, const void* left,
                       const void* right, double cs, void* flux, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (rsolver < JX_LLF || rsolver > JX_ROE) return fail(JX_ERR_UNSUPPORTED, "unknown Riemann solver %d", rsolver);
  if (axis != 0 && axis != 1) return fail(JX_ERR_INVALID, "axis must be 0 (y) or 1 (x)");
  if (nface < 0 || nv < 3) return fail(JX_ERR_INVALID, "bad shape");
  if (nface > 0 && (!left || !right || !flux)) return fail(JX_ERR_INVALID, "null array");
  return cuda_check(launch_face_flux(dtype, rsolver, nface, nv, axis, left, right, cs, flux, (cudaStream_t)s),
                    "face-flux kernel");
}

jx_status jx_viscous_flux(int32_t dtype, int32_t ny, int32_t nx, int32_t nv, const void* W, double dx, double dy,
                          double viscosity, double smagorinsky_cs, int32_t axis, void* out, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (axis != 0 && axis != 1) return fail(JX_ERR_INVALID, "axis must be 0 (y) or 1 (x)");
  if (ny < 0 || nx < 0 || nv < 3) return fail(JX_ERR_INVALID, "bad shape");
  if ((int64_t)ny * nx > 0 && (!W || !out)) return fail(JX_ERR_INVALID, "null array");
  return cuda_check(launch_viscous_flux(dtype, ny, nx, nv, W, dx, dy, viscosity, smagorinsky_cs, axis, out,
                                        (cudaStream_t)s),
                    "viscous-flux kernel");
}

jx_status jx_face_velocity_gradients(int32_t dtype, int32_t ny, int32_t nx, int32_t nv, const void* W, double dx,
                                     double dy, int32_t axis, void* dv_dx, void* dv_dy, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (axis != 0 && axis != 1) return fail(JX_ERR_INVALID, "axis must be 0 (y) or 1 (x)");
  if (ny < 0 || nx < 0 || nv < 3) return fail(JX_ERR_INVALID, "bad shape");
  if ((int64_t)ny * nx > 0 && (!W || !dv_dx || !dv_dy)) return fail(JX_ERR_INVALID, "null array");
  return cuda_check(launch_face_gradients(dtype, ny, nx, nv, W, dx, dy, axis, dv_dx, dv_dy, (cudaStream_t)s),
                    "face-gradient kernel");
}

jx_status jx_smagorinsky_viscosity(int32_t dtype, int64_t ncell, const void* dv_dx, const void* dv_dy, double dx,
                                   double dy, double smagorinsky_cs, void* out, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (ncell < 0 || (ncell > 0 && (!dv_dx || !dv_dy || !out))) return fail(JX_ERR_INVALID, "bad arguments");
  const double c = smagorinsky_cs * smagorinsky_cs * dx * dy;
  return cuda_check(launch_smagorinsky(dtype, ncell, dv_dx, dv_dy, c, out, (cudaStream_t)s), "Smagorinsky kernel");
}

jx_status jx_probe_fma(int32_t dtype, int32_t blocks, int32_t iters, int32_t chains, double* sink, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (blocks < 1 || iters < 1 || !sink || (chains != 8 && chains != 16 && chains != 32))
    return fail(JX_ERR_INVALID, "bad probe arguments");
  return cuda_check(launch_probe(dtype, blocks, iters, chains, sink, (cudaStream_t)s), "probe kernel");
}

jx_status jx_probe_math(int32_t dtype, int64_t n, const void* a, const void* b, void* rcp_out, void* div_out,
                        void* geo_out, jx_stream s) {
  if (dtype != JX_F64 && dtype != JX_F32) return fail(JX_ERR_UNSUPPORTED, "unknown dtype %d", dtype);
  if (n < 0 || (n > 0 && (!a || !b || !rcp_out || !div_out || !geo_out)))
    return fail(JX_ERR_INVALID, "bad probe arguments");
  return cuda_check(launch_math_probe(dtype, n, a, b, rcp_out, div_out, geo_out, (cudaStream_t)s),
                    "math probe kernel");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many solves advanced together, one persistent stage launch per
// (precision, reconstruction, Riemann solver) group and RK stage.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t kPlanMagic = 0x4a584250;  // "JXBP"
// 2 precisions x 5 reconstructions x 3 solvers x 19 kernel classes (shared
// memory; marching with 3 or 4 variables at 1, 2 or 3 columns per lane, with
// or without the row ring; lean 4-variable two-column groups per integrator,
// with or without the ring)
constexpr int kMaxGroups = 570;

struct BatchGroup {
  int dtype, recon, rsolver, first, count, tile_first, nwork, march;
  int nv;   // marching groups: the variable count of every solve (0 in shared-memory groups)
  int nc;   // marching groups: columns per lane (0 in shared-memory groups)
  int ring;  // marching groups: tiles of kRingMinRows rows or more, where a ring kernel runs
  int lean;  // marching groups of inviscid 4-variable float32 solves with one integrator
  int integrator;  // lean groups: the members' integrator (-1 otherwise)
  int form[4];     // lean groups: the MarchForm of each stage
  int bps;  // resident blocks per SM of the group's kernel (occupancy at plan time)
  size_t smem;
};

struct BatchSolveInfo {
  jx_solve solve;  // with desc.tile_x/tile_y set to the plan's tile
  int forced, smag, n_stages, pad;
};

// Forced solves of one precision: their render and kick parameters sit at
// [first, first + count) of the plan's force arrays; block offsets of the
// render, the two sum passes and the kick at [off, off + count + 1) of the
// three offset arrays.
struct ForceGroup {
  int dtype, first, count, off;
  int render_work, sum_work, kick_work, pad;
};

struct BatchPlanHeader {
  uint32_t magic;
  int32_t n, n_groups, max_stages, n_force_groups;
  int64_t bytes, off_params, off_offsets, off_begin, off_info;
  int64_t off_force, off_render, off_force_offsets;
  BatchGroup groups[kMaxGroups];
  ForceGroup force_groups[2];
};

struct PlanLayout {
  size_t params, offsets, begin, info, force, render, force_offsets, total;
};

PlanLayout plan_layout(int n) {
  PlanLayout L;
  size_t off = align256(sizeof(BatchPlanHeader));
  L.params = off;
  off = align256(off + (size_t)4 * n * sizeof(StageParams));
  L.offsets = off;
  off = align256(off + (size_t)(n + kMaxGroups) * sizeof(int));
  L.begin = off;
  off = align256(off + (size_t)n * sizeof(BeginParams));
  L.info = off;
  off = align256(off + (size_t)n * sizeof(BatchSolveInfo));
  L.force = off;
  off = align256(off + (size_t)n * sizeof(ForceParams));
  L.render = off;
  off = align256(off + (size_t)n * sizeof(RenderParams));
  L.force_offsets = off;
  off = align256(off + (size_t)3 * (n + 2) * sizeof(int));
  L.total = off;
  return L;
}

int sm_count() {
  static int sms[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!sms[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sms[dev] = v > 0 ? v : 1;
  }
  return sms[dev];
}

int batch_occupancy(int recon, int dtype, int rsolver, size_t smem) {
  switch (recon) {
    case JX_DC: return batch_blocks_per_sm_dc(dtype, rsolver, smem);
    case JX_PLM: return batch_blocks_per_sm_plm(dtype, rsolver, smem);
    case JX_PPM4: return batch_blocks_per_sm_ppm4(dtype, rsolver, smem);
    case JX_PPMX: return batch_blocks_per_sm_ppmx(dtype, rsolver, smem);
    default: return batch_blocks_per_sm_wenoz(dtype, rsolver, smem);
  }
}

cudaError_t launch_batch(int recon, int dtype, int rsolver, const StageParams* params, const int* offsets,
                         int nsolves, int nwork, dim3 grid, size_t smem, cudaStream_t s) {
  switch (recon) {
    case JX_DC: return launch_batch_dc(dtype, rsolver, params, offsets, nsolves, nwork, grid, smem, s);
    case JX_PLM: return launch_batch_plm(dtype, rsolver, params, offsets, nsolves, nwork, grid, smem, s);
    case JX_PPM4: return launch_batch_ppm4(dtype, rsolver, params, offsets, nsolves, nwork, grid, smem, s);
    case JX_PPMX: return launch_batch_ppmx(dtype, rsolver, params, offsets, nsolves, nwork, grid, smem, s);
    default: return launch_batch_wenoz(dtype, rsolver, params, offsets, nsolves, nwork, grid, smem, s);
  }
}

int batch_march_occupancy(int recon, int dtype, int rsolver, int nv, int nc, int ring, int lean) {
  const int kind = lean ? (ring ? kMarchBatchPackedRing : kMarchBatchPacked) : (ring ? kMarchBatchRing : kMarchBatch);
  switch (recon) {
    case JX_DC: return march_blocks_per_sm_dc(dtype, rsolver, nv, nc, kind);
    case JX_PLM: return march_blocks_per_sm_plm(dtype, rsolver, nv, nc, kind);
    case JX_PPM4: return march_blocks_per_sm_ppm4(dtype, rsolver, nv, nc, kind);
    case JX_PPMX: return march_blocks_per_sm_ppmx(dtype, rsolver, nv, nc, kind);
    default: return march_blocks_per_sm_wenoz(dtype, rsolver, nv, nc, kind);
  }
}

cudaError_t launch_batch_march(int recon, int dtype, int rsolver, int nv, int nc, int ring, int form,
                               const StageParams* params, const int* offsets, int nsolves, int nwork, dim3 grid,
                               cudaStream_t s) {
  switch (recon) {
    case JX_DC: return launch_batch_march_dc(dtype, rsolver, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
    case JX_PLM: return launch_batch_march_plm(dtype, rsolver, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
    case JX_PPM4: return launch_batch_march_ppm4(dtype, rsolver, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
    case JX_PPMX: return launch_batch_march_ppmx(dtype, rsolver, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
    default: return launch_batch_march_wenoz(dtype, rsolver, nv, nc, ring, form, params, offsets, nsolves, nwork, grid, s);
  }
}

// Side streams of one device for the concurrent stage groups of a batch step;
// the returned lock serialises batch steps of different host threads on them
// (the fork and join events are shared).
constexpr int kSideStreams = 8;

struct SideStreams {
  cudaStream_t s[kSideStreams];
  cudaEvent_t fork, join[kSideStreams];
  bool ready;
};

std::mutex g_side_mutex[64];
SideStreams g_side[64];

jx_status side_streams(SideStreams** out, std::unique_lock<std::mutex>* lock) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(JX_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(JX_ERR_INVALID, "device ordinal %d out of range", dev);
  *lock = std::unique_lock<std::mutex>(g_side_mutex[dev]);
  SideStreams& S = g_side[dev];
  if (!S.ready) {
    for (int k = 0; k < kSideStreams && e == cudaSuccess; ++k) e = cudaStreamCreateWithFlags(&S.s[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S.fork, cudaEventDisableTiming);
    for (int k = 0; k < kSideStreams && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&S.join[k], cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(JX_ERR_CUDA, "side streams: %s", cudaGetErrorString(e));
    S.ready = true;
  }
  *out = &S;
  return JX_OK;
}

jx_status check_batch_solve(int i, const jx_solve& in, Tile* t, Ws* w) {
  jx_status st = check_desc(&in.desc);
  if (st) return fail(st, "solve %d: %s", i, jx_last_error());
  const jx_desc& d = in.desc;
  if (d.nvar != 3 && d.nvar != 4) return fail(JX_ERR_INVALID, "solve %d: batches take 3 or 4 variables", i);
  if (!in.S || !in.A || !in.B || !in.clock) return fail(JX_ERR_INVALID, "solve %d: null state or clock", i);
  if (in.S == in.A || in.S == in.B || in.A == in.B) return fail(JX_ERR_INVALID, "solve %d: S, A, B must differ", i);
  if (d.nvar == 4 && !(aligned16(in.S) && aligned16(in.A) && aligned16(in.B)))
    return fail(JX_ERR_INVALID, "solve %d: 4-variable states must be 16-byte aligned", i);
  if ((st = resolve_tile(&d, t))) return fail(st, "solve %d: %s", i, jx_last_error());
  if (!t->march && !t->fast_shape)
    return fail(JX_ERR_INVALID, "solve %d: batch tiles are 32 x h or 26/58/90 x h, not %d x %d", i, t->tx, t->ty);
  if (!t->march && t->ty > 64) return fail(JX_ERR_INVALID, "solve %d: batch tiles have at most 64 rows", i);
  if ((st = bind_ws(&d, *t, in.workspace, in.workspace_bytes, w))) return fail(st, "solve %d: %s", i, jx_last_error());
  if (in.forcing.raw_force && (!in.forcing.table || !in.forcing.cos_x || !in.forcing.sin_x || !in.forcing.cos_y ||
                               !in.forcing.sin_y || in.forcing.n_modes < 1 || in.forcing.n_updates < 1))
    return fail(JX_ERR_INVALID, "solve %d: incomplete forcing tables", i);
  return JX_OK;
}

}  // namespace

extern "C" {

jx_status jx_batch_plan_bytes(const jx_solve* solves, int32_t n, size_t* bytes) {
  if (!solves || n < 1 || !bytes) return fail(JX_ERR_INVALID, "a batch needs at least one solve");
  *bytes = plan_layout(n).total;
  return JX_OK;
}

jx_status jx_batch_plan(const jx_solve* solves, int32_t n, void* plan, size_t bytes) {
  size_t need = 0;
  jx_status st = jx_batch_plan_bytes(solves, n, &need);
  if (st) return st;
  if (!plan || bytes < need) return fail(JX_ERR_WORKSPACE, "plan buffer has %zu bytes, needs %zu", bytes, need);
  const PlanLayout L = plan_layout(n);
  char* base = static_cast<char*>(plan);
  memset(base, 0, need);
  BatchPlanHeader* h = reinterpret_cast<BatchPlanHeader*>(base);
  h->magic = kPlanMagic;
  h->n = n;
  h->bytes = (int64_t)need;
  h->off_params = (int64_t)L.params;
  h->off_offsets = (int64_t)L.offsets;
  h->off_begin = (int64_t)L.begin;
  h->off_info = (int64_t)L.info;
  h->off_force = (int64_t)L.force;
  h->off_render = (int64_t)L.render;
  h->off_force_offsets = (int64_t)L.force_offsets;
  StageParams* params = reinterpret_cast<StageParams*>(base + L.params);
  int* offsets = reinterpret_cast<int*>(base + L.offsets);
  BeginParams* begin = reinterpret_cast<BeginParams*>(base + L.begin);
  BatchSolveInfo* info = reinterpret_cast<BatchSolveInfo*>(base + L.info);

  // Validate every solve once, then group by (precision, reconstruction,
  // Riemann solver, kernel; and variable count for the marching kernel,
  // which is compiled per count) in order of first appearance; solves keep
  // their relative order inside a group. A shared-memory group launches with
  // the largest tile of its solves; each solve walks its own tiles.
  std::vector<jx_solve> sv(solves, solves + n);
  std::vector<Tile> tl(n);
  std::vector<Ws> wl(n);
  for (int i = 0; i < n; ++i)
    if ((st = check_batch_solve(i, solves[i], &tl[i], &wl[i]))) return st;
  std::vector<int> group_of(n, -1);
  int n_groups = 0;
  for (int i = 0; i < n; ++i) {
    const jx_desc& d = sv[i].desc;
    const int march = tl[i].march ? 1 : 0;
    const int nv = march ? d.nvar : 0;
    const int nc = march ? tl[i].mnc : 0;
    // Lean groups (no viscosity, Smagorinsky or drag; 4 variables, two
    // columns per lane, float32; one integrator, so every member's stage has
    // the same form) may run the packed walk, with or without the ring.
    const int lean = march && d.dtype == JX_F32 && d.nvar == 4 && nc == 2 && d.viscosity == 0.0 &&
                     d.smagorinsky_cs == 0.0 && d.drag_rate == 0.0;
    const int integrator = lean ? d.integrator : -1;
    const int ring = march && tl[i].mty >= kRingMinRows && (lean || march_ring_built(d.dtype == JX_F32, d.recon, nc));
    int g = 0;
    while (g < n_groups && !(h->groups[g].dtype == d.dtype && h->groups[g].recon == d.recon &&
                             h->groups[g].rsolver == d.rsolver && h->groups[g].march == march &&
                             h->groups[g].nv == nv && h->groups[g].nc == nc && h->groups[g].ring == ring &&
                             h->groups[g].lean == lean && h->groups[g].integrator == integrator))
      ++g;
    if (g == n_groups) {
      if (n_groups == kMaxGroups) return fail(JX_ERR_INVALID, "more than %d solver groups", kMaxGroups);
      BatchGroup& G = h->groups[n_groups++];
      G.dtype = d.dtype;
      G.recon = d.recon;
      G.rsolver = d.rsolver;
      G.march = march;
      G.nv = nv;
      G.nc = nc;
      G.ring = ring;
      G.lean = lean;
      G.integrator = integrator;
      for (int k = 0; k < 4; ++k) G.form[k] = kMarchGeneric;
      G.smem = 0;
    }
    if (!march && tl[i].fast_smem > h->groups[g].smem) h->groups[g].smem = tl[i].fast_smem;
    group_of[i] = g;
  }
  int order_count = 0, next_int = 0;
  for (int g = 0; g < n_groups; ++g) {
    BatchGroup& G = h->groups[g];
    G.first = order_count;
    G.tile_first = next_int;
    int tiles = 0;
    for (int i = 0; i < n; ++i) {
      if (group_of[i] != g) continue;
      const jx_desc& d = sv[i].desc;
      const Tile& t = tl[i];
      const Ws& w = wl[i];
      const int k = order_count++;
      const int nst = jx_num_stages(d.integrator);
      const bool forced = sv[i].forcing.raw_force != nullptr;
      BatchSolveInfo& I = info[k];
      I.solve = sv[i];
      I.forced = forced;
      I.smag = d.smagorinsky_cs > 0.0;
      I.n_stages = nst;
      if (nst > h->max_stages) h->max_stages = nst;
      offsets[next_int++] = tiles;
      tiles += G.march ? t.mtiles_x * t.mtiles_y : t.tiles_x * t.tiles_y;
      BeginParams& B = begin[k];
      B.q = dt_params(&d);
      B.clock = sv[i].clock;
      B.partials = w.cfl;
      B.header = w.header;
      B.forced = forced;
      const void* in = sv[i].S;
      for (int stage = 1; stage <= 4; ++stage) {
        StageParams& P = params[(size_t)(stage - 1) * n + k];
        if (stage > nst) {
          memset(&P, 0, sizeof(P));
          P.skip = 1;
          P.clock = sv[i].clock;
          continue;
        }
        void* out = stage == nst ? sv[i].S : (stage % 2 == 1 ? sv[i].A : sv[i].B);
        P = make_stage_params(&d, t, w, stage, in, sv[i].S, out, stage == nst ? nullptr : sv[i].S, nullptr,
                              forced, sv[i].clock, nullptr);
        if (G.march) {
          P.tx = march_tile_x(t.mnc);
          P.nc = t.mnc;
          P.ty = t.mty;
          P.tiles_x = t.mtiles_x;
          if (G.lean) G.form[stage - 1] = P.blend ? kMarchLeanBlend : kMarchLeanPlain;
        }
        in = out;
      }
    }
    offsets[next_int++] = tiles;
    G.count = order_count - G.first;
    G.nwork = tiles;
  }
  h->n_groups = n_groups;
  for (int g = 0; g < n_groups; ++g) {
    BatchGroup& G = h->groups[g];
    G.bps = G.march ? batch_march_occupancy(G.recon, G.dtype, G.rsolver, G.nv, G.nc, G.ring, G.lean)
                    : batch_occupancy(G.recon, G.dtype, G.rsolver, G.smem);
    if (G.bps < 1) {
      cudaGetLastError();  // no device to query: one block per SM
      G.bps = 1;
    }
  }

  // Forced solves, grouped by precision, for the batched render and kick.
  ForceParams* fq = reinterpret_cast<ForceParams*>(base + L.force);
  RenderParams* rq = reinterpret_cast<RenderParams*>(base + L.render);
  int* foff = reinterpret_cast<int*>(base + L.force_offsets);
  int* off_render = foff;
  int* off_sum = foff + (n + 2);
  int* off_kick = foff + 2 * (n + 2);
  int nf = 0, next_off = 0;
  for (int dt = JX_F64; dt <= JX_F32; ++dt) {
    ForceGroup F;
    memset(&F, 0, sizeof(F));
    F.dtype = dt;
    F.first = nf;
    F.off = next_off;
    for (int k = 0; k < n; ++k) {
      const BatchSolveInfo& I = info[k];
      if (!I.forced || I.solve.desc.dtype != dt) continue;
      const jx_desc& d = I.solve.desc;
      Tile t;
      Ws w;
      if ((st = resolve_tile(&d, &t)) || (st = bind_ws(&d, t, I.solve.workspace, I.solve.workspace_bytes, &w)))
        return st;
      fq[nf] = force_params(&d, &I.solve.forcing, I.solve.S, I.solve.clock, nullptr, w);
      rq[nf] = render_params(&d, &I.solve.forcing, I.solve.clock);
      const int64_t ncell = (int64_t)d.ny * d.nx;
      off_render[next_off] = F.render_work;
      off_sum[next_off] = F.sum_work;
      off_kick[next_off] = F.kick_work;
      F.render_work += render_blocks(d.ny, d.nx);
      F.sum_work += fq[nf].nblk;
      F.kick_work += kick_blocks(ncell);
      ++next_off;
      ++nf;
      ++F.count;
    }
    if (F.count == 0) continue;
    off_render[next_off] = F.render_work;
    off_sum[next_off] = F.sum_work;
    off_kick[next_off] = F.kick_work;
    ++next_off;
    h->force_groups[h->n_force_groups++] = F;
  }
  return JX_OK;
}

jx_status jx_batch_step(const void* plan, const void* plan_dev, int32_t blocks_per_sm, jx_stream stream) {
  const BatchPlanHeader* h = static_cast<const BatchPlanHeader*>(plan);
  if (!h || !plan_dev || h->magic != kPlanMagic) return fail(JX_ERR_INVALID, "not a batch plan");
  cudaStream_t s = (cudaStream_t)stream;
  const char* base = static_cast<const char*>(plan);
  const char* dbase = static_cast<const char*>(plan_dev);
  const BatchSolveInfo* info = reinterpret_cast<const BatchSolveInfo*>(base + h->off_info);
  const StageParams* params_dev = reinterpret_cast<const StageParams*>(dbase + h->off_params);
  const int* offsets_dev = reinterpret_cast<const int*>(dbase + h->off_offsets);
  const BeginParams* begin_dev = reinterpret_cast<const BeginParams*>(dbase + h->off_begin);
  jx_status st;
  if ((st = cuda_check(launch_begin_step_batch(begin_dev, h->n, s), "batched begin-step kernel"))) return st;
  const ForceParams* force_dev = reinterpret_cast<const ForceParams*>(dbase + h->off_force);
  const RenderParams* render_dev = reinterpret_cast<const RenderParams*>(dbase + h->off_render);
  const int* foff_dev = reinterpret_cast<const int*>(dbase + h->off_force_offsets);
  for (int g = 0; g < h->n_force_groups; ++g) {
    const ForceGroup& F = h->force_groups[g];
    if ((st = cuda_check(launch_render_batch(F.dtype, render_dev + F.first, foff_dev + F.off, F.count,
                                             F.render_work, s),
                         "batched render kernel")))
      return st;
  }
  // A stage's launch groups are independent (disjoint solves): with more
  // than one they run concurrently on side streams that fork from and join
  // back to the caller's stream around each stage (also inside a graph
  // capture), so small groups do not wait for one another.
  const int sms = sm_count();
  SideStreams* side = nullptr;
  std::unique_lock<std::mutex> side_lock;
  if (h->n_groups > 1 && (st = side_streams(&side, &side_lock))) return st;
  for (int stage = 1; stage <= h->max_stages; ++stage) {
    const int used = side ? (h->n_groups < kSideStreams ? h->n_groups : kSideStreams) : 0;
    if (side) {
      if ((st = cuda_check(cudaEventRecord(side->fork, s), "fork event"))) return st;
      for (int k = 0; k < used; ++k)
        if ((st = cuda_check(cudaStreamWaitEvent(side->s[k], side->fork, 0), "side stream wait"))) return st;
    }
    for (int g = 0; g < h->n_groups; ++g) {
      const BatchGroup& G = h->groups[g];
      int bps = blocks_per_sm;
      if (bps <= 0) bps = G.bps;
      if (bps < 1) bps = 1;
      int64_t blocks = (int64_t)sms * bps;
      const int64_t per_block = G.march ? kMarchWarps : 1;  // marching blocks take one tile per warp
      if (blocks > (G.nwork + per_block - 1) / per_block) blocks = (G.nwork + per_block - 1) / per_block;
      if (blocks < 1) continue;
      const StageParams* P = params_dev + (size_t)(stage - 1) * h->n + G.first;
      const int* offs = offsets_dev + G.tile_first;
      cudaStream_t gs = side ? side->s[g % kSideStreams] : s;
      const cudaError_t e =
          G.march ? launch_batch_march(G.recon, G.dtype, G.rsolver, G.nv, G.nc, G.ring,
                                       G.lean ? G.form[stage - 1] : kMarchGeneric, P, offs, G.count, G.nwork,
                                       dim3((unsigned)blocks), gs)
                  : launch_batch(G.recon, G.dtype, G.rsolver, P, offs, G.count, G.nwork, dim3((unsigned)blocks),
                                 G.smem, gs);
      if ((st = cuda_check(e, "batched stage kernel"))) return st;
    }
    for (int k = 0; k < used; ++k) {
      if ((st = cuda_check(cudaEventRecord(side->join[k], side->s[k]), "join event"))) return st;
      if ((st = cuda_check(cudaStreamWaitEvent(s, side->join[k], 0), "join wait"))) return st;
    }
  }
  for (int g = 0; g < h->n_force_groups; ++g) {
    const ForceGroup& F = h->force_groups[g];
    const int* off_sum = foff_dev + (h->n + 2) + F.off;
    const int* off_kick = foff_dev + 2 * (h->n + 2) + F.off;
    if ((st = cuda_check(launch_force_kick_batch(F.dtype, force_dev + F.first, F.count, off_sum, F.sum_work, off_kick,
                                                 F.kick_work, s),
                         "batched force kick kernels")))
      return st;
  }
  for (int i = 0; i < h->n; ++i) {
    const jx_solve& sv = info[i].solve;
    if (!info[i].smag) continue;
    Tile t;
    Ws w;
    if ((st = resolve_tile(&sv.desc, &t)) || (st = bind_ws(&sv.desc, t, sv.workspace, sv.workspace_bytes, &w)))
      return st;
    CflParams q = cfl_params(&sv.desc, sv.S, sv.clock, w);
    if ((st = cuda_check(launch_cfl(sv.desc.dtype, false, q, s), "cfl kernel"))) return st;
  }
  return JX_OK;
}

int32_t jx_batch_groups(const void* plan) {
  const BatchPlanHeader* h = static_cast<const BatchPlanHeader*>(plan);
  return h && h->magic == kPlanMagic ? h->n_groups : -1;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// jx_timestep_noalloc: isothermal_timestep for callers that cannot allocate
// device memory and have no workspace to pass.
//
// Its scratch is g_timestep_scratch below: a file-scope device array that
// holds the per-block CFL partials and their count. The CFL kernel launches at
// most kCflBlocksMax blocks and strides over larger grids, so 2048 partial
// slots (64 KiB + a 256-byte header) cover every grid jx_check_desc accepts.
// Every GPU that loads libjx.so keeps these 65,792 bytes until the process
// exits. All calls share the array: each call rewrites every slot it reads
// (the count included) before reading it, so nothing has to start at zero,
// but two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on the array.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocSlots = jx::kCflBlocksMax;
constexpr size_t kNoAllocBytes = jx::kWsHeader + kNoAllocSlots * jx::kCflSlots * sizeof(double);
// cfl_grid() never launches more than kCflBlocksMax blocks, so every grid fits.
static_assert(kNoAllocSlots >= (size_t)jx::kCflBlocksMax, "timestep scratch must hold every CFL partial");
static __device__ __align__(256) unsigned char g_timestep_scratch[kNoAllocBytes];

std::mutex g_scratch_mutex;
void* g_scratch_address[64] = {};  // device address of g_timestep_scratch, per device

// The array's host-side name is not a device address; look the address up
// once per device, with that device current.
jx_status scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(JX_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(JX_ERR_INVALID, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_address[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_timestep_scratch);
    if (e != cudaSuccess || !p)
      return fail(JX_ERR_CUDA, "cudaGetSymbolAddress(timestep scratch): %s", cudaGetErrorString(e));
    g_scratch_address[dev] = p;
  }
  *out = g_scratch_address[dev];
  return JX_OK;
}

}  // namespace

extern "C" jx_status jx_timestep_noalloc(const jx_desc* d, const void* W, double cfl, double prev_dt,
                                         double time, double tlim, double* dt_out, jx_stream s) {
  jx_status st = check_desc(d);
  if (st) return st;
  if (!W || !dt_out) return fail(JX_ERR_INVALID, "null W or dt_out");
  // The same descriptors as jx_timestep: an explicit tile it would refuse
  // (too much shared memory, too few marching rows) is refused here too.
  Tile t;
  if ((st = resolve_tile(d, &t, false))) return st;
  const int64_t ncell = (int64_t)d->ny * d->nx;
  const size_t need = kWsHeader + (size_t)cfl_grid(ncell) * kCflSlots * sizeof(double);
  // Unreachable while cfl_grid caps its blocks (static_assert above); kept so
  // that a change to that cap fails loudly instead of overrunning the array.
  if (need > kNoAllocBytes)
    return fail(JX_ERR_INVALID, "grid of %lld cells needs %zu bytes of timestep scratch; the static scratch holds %zu",
                (long long)ncell, need, kNoAllocBytes);
  void* base = nullptr;
  if ((st = scratch_address(&base))) return st;
  Ws w;
  w.header = static_cast<WsHeader*>(base);
  w.cfl = reinterpret_cast<double*>(static_cast<char*>(base) + kWsHeader);
  CflParams q = cfl_params(d, W, nullptr, w);
  if ((st = cuda_check(launch_cfl(d->dtype, true, q, (cudaStream_t)s), "cfl kernel"))) return st;
  return cuda_check(launch_timestep_finish(dt_params(d), w.cfl, w.header, prev_dt, time, tlim, cfl, dt_out,
                                           (cudaStream_t)s),
                    "timestep finisher");
}
