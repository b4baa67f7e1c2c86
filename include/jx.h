/*
 * jx.h — C ABI of libjx.so, the GB300 (sm_103a) implementation of JathenAX's
 * per-Runge-Kutta-stage isothermal hydro right-hand side.
 *
 * Conventions
 *   - Every buffer is caller-owned device memory. State arrays are
 *     (ny, nx, nvar) row-major with the component innermost
 *     (rho, rho*vx, rho*vy, rho*s1, ...), the layout of the reference's npz
 *     files and of its `U` arrays (jathenax/run.py:184-185).
 *   - Calls are stream-ordered and never synchronise the host, allocate, or
 *     abort. They return JX_OK (0) or a negative jx_status; jx_last_error()
 *     returns a message for the calling thread's last failure.
 *   - `jx_clock` is a small device-resident struct that carries time, dt,
 *     cycle and the forcing schedule between kernels so a whole step can be
 *     enqueued (or captured in a CUDA graph) without a host round trip.
 *
 * Each entry point names the reference function it replaces (file:line in
 * the JathenAX source tree).
 */
#ifndef JX_H
#define JX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* jx_stream; /* a cudaStream_t; NULL = legacy default stream */

typedef enum {
  JX_OK = 0,
  JX_ERR_INVALID = -1,     /* bad argument (reference raises ValueError)  */
  JX_ERR_UNSUPPORTED = -2, /* selector not known (reference raises KeyError) */
  JX_ERR_CUDA = -3,        /* a CUDA launch or copy failed                  */
  JX_ERR_WORKSPACE = -4    /* workspace too small or misaligned             */
} jx_status;

typedef enum { JX_F64 = 0, JX_F32 = 1 } jx_dtype;
/* fluxes.py:120-123 RECONSTRUCTIONS */
typedef enum { JX_DC = 0, JX_PLM = 1, JX_PPM4 = 2, JX_PPMX = 3, JX_WENOZ = 4 } jx_recon;
/* fluxes.py:204 RIEMANN_SOLVERS */
typedef enum { JX_LLF = 0, JX_HLLE = 1, JX_ROE = 2 } jx_rsolver;
/* hydro.py:20-36 RK_STAGES */
typedef enum { JX_RK2 = 0, JX_RK3 = 1, JX_RK4 = 2 } jx_integrator;

/* Problem description: the static arguments of isothermal_step
 * (hydro.py:92-95) and evolve_isothermal (run.py:24-27). */
typedef struct {
  int32_t ny, nx, nvar;   /* nvar >= 3; components 3.. are passive scalars */
  int32_t dtype;          /* jx_dtype */
  int32_t recon, rsolver, integrator;
  /* Stage tile. 0, 0 = library default: for 3/4 variables, float32 uses
   * the register-marching kernel (58 x h tiles, 26 x h for WENO-Z, h
   * chosen per device and grid) and float64 32 x 16 shared-memory tiles.
   * tile_x = 26, 58 or 90 selects marching tiles for 3/4 variables
   * (tile_y >= 8 rows, or 0 for automatic). Any other tile_x x tile_y is a
   * shared-memory tile. See jx_tile_info. */
  int32_t tile_x, tile_y;
  double dx, dy, cs, dfloor;
  double viscosity, smagorinsky_cs, drag_rate;
} jx_desc;

/* Device-resident step control (run.py:63-69 loop state). The host writes
 * it once (time 0, prev_dt inf, cycle 0, update -1, tlim/nlim/cfl and the
 * forcing schedule) and reads it back when `done` is set. */
typedef struct {
  double time, dt, prev_dt, tlim;
  double cfl, power, t_start, dt_update;
  double dedt, reserved0, reserved1, reserved2;
  int32_t cycle, nlim, update, render;
  int32_t done, pending, n_updates, status;
} jx_clock;

/* Turbulence driver tables (forcing.py:63-122), device pointers. The phase
 * tables and the raw-force buffer are in the state dtype; the OU table is
 * float64 [n_updates][n_modes][2 dir][2 re/im] in either precision. */
typedef struct {
  const double* table;
  const void* cos_x; const void* sin_x; /* [n_modes][nx] */
  const void* cos_y; const void* sin_y; /* [n_modes][ny] */
  void* raw_force;                      /* (ny, nx, 2) cached raw acceleration */
  int32_t n_updates, n_modes;
} jx_forcing;

/* Optional per-stage outputs of hydro.py:135-142 (trace=True). Any pointer
 * may be NULL. left/right/flux are (ny, nx, nvar) at the low face of each
 * cell; primitives is (ny, nx, nvar); saved/conserved as in the reference. */
typedef struct {
  void *primitives, *left_x, *right_x, *left_y, *right_y, *flux_x, *flux_y;
  void *saved, *conserved;
  void *before_kick;  /* (ny, nx, nvar), final stage of a forced step only */
  void *acceleration; /* (ny, nx, 2),    final stage of a forced step only */
} jx_trace;

/* Message for the calling thread's last failing call ("" if none). */
const char* jx_last_error(void);
/* Library version string. */
const char* jx_version(void);

/* Bytes of device workspace the stage/step/timestep calls need for `d`.
 * The workspace must be 256-byte aligned. */
jx_status jx_workspace_bytes(const jx_desc* d, size_t* bytes);
/* Validate `d` (sizes, selectors, finite coefficients). */
jx_status jx_check_desc(const jx_desc* d);
/* Number of RK stages of d->integrator (hydro.py:20-36). */
int32_t jx_num_stages(int32_t integrator);

/* recover_isothermal (hydro.py:54-60): floor rho into U_out and write
 * W = (rho, m/rho, (rho s)/rho). U_out or W may be NULL. */
jx_status jx_recover(const jx_desc* d, const void* U, void* U_out, void* W, jx_stream s);

/* isothermal_timestep (hydro.py:63-89) on primitives W (ny, nx, nvar):
 * writes dt (float64) to *dt_out (device). prev_dt/time/tlim are host values. */
jx_status jx_timestep(const jx_desc* d, const void* W, double cfl, double prev_dt,
                      double time, double tlim, double* dt_out, void* workspace,
                      size_t workspace_bytes, jx_stream s);

/* isothermal_timestep without a workspace, for callers that cannot allocate
 * device memory: e.g. a JAX/XLA FFI handler, where XLA has reserved most of
 * the GPU and owns every buffer, or a loop with a no-allocation rule. No
 * counterpart in the reference (which never allocates explicitly).
 * Same arguments and result as jx_timestep minus the workspace. Its scratch
 * is a 65,792-byte static device array in libjx.so (2048 CFL partial slots,
 * enough for every grid jx_check_desc accepts; a grid that needed more would
 * be refused with JX_ERR_INVALID). The first call on a device looks up the
 * array's address on that device; make that first call before any stream
 * capture. The address is kept per device for the life of the process: after
 * cudaDeviceReset (which unloads the library's device code) it is stale, so
 * do not call this entry point on a device that has been reset. Calls share
 * the array: calls whose kernels overlap on the GPU race. Allocates nothing. */
jx_status jx_timestep_noalloc(const jx_desc* d, const void* W, double cfl, double prev_dt,
                              double time, double tlim, double* dt_out, jx_stream s);

/* One RK stage of isothermal_step (hydro.py:101-143) fused into one kernel:
 * reconstruction, Riemann solve, viscous + Smagorinsky + SGS stress, flux
 * divergence, the RK combine (rk_stage, hydro.py:39-51), drag, and the
 * density floor. stage is 1-based. U_in is read with its halo; V_in, V_out
 * and U_out are read/written only at each cell, so V_in, V_out and U_out
 * may alias each other but not U_in. tau (ny, nx, 3) or NULL is the SGS
 * stress. dt is read from clock->dt. On the last stage the kernel also
 * writes CFL partials for jx_begin_step. If `force_follows` the last stage
 * leaves U_out unfloored for jx_force_kick. trace may be NULL. */
jx_status jx_stage(const jx_desc* d, int32_t stage, const void* U_in, const void* V_in,
                   void* U_out, void* V_out, const void* tau, int32_t force_follows,
                   jx_clock* clock, const jx_trace* trace, void* workspace,
                   size_t workspace_bytes, jx_stream s);

/* CFL / Smagorinsky partials of the conserved state U (hydro.py:63-80 with
 * W = recover(U)); needed before the first jx_begin_step, and after each
 * step when smagorinsky_cs > 0 (the fused stage kernel cannot see the new
 * state's face gradients). */
jx_status jx_cfl_partials(const jx_desc* d, const void* U, void* workspace,
                          size_t workspace_bytes, jx_stream s);

/* Start of one evolve_isothermal cycle (run.py:40-53): commit the previous
 * cycle's time/cycle, stop (clock->done) at tlim or nlim, pick dt from the
 * CFL partials (hydro.py:63-89) and decide whether the forcing field must be
 * re-rendered (forcing.py:125-134). `forced` selects the forcing schedule. */
jx_status jx_begin_step(const jx_desc* d, jx_clock* clock, int32_t forced, void* workspace,
                        size_t workspace_bytes, jx_stream s);

/* render_force/update_force (forcing.py:111-134): re-render f->raw_force from
 * table row clock->update when clock->render is set. */
jx_status jx_force_render(const jx_desc* d, const jx_forcing* f, jx_clock* clock, jx_stream s);

/* normalize_force + kick + recovery (forcing.py:137-149, hydro.py:128-143) on
 * the final stage's unfloored U, in place, followed by CFL partials of the
 * kicked state. The kick uses clock->dt and clock->power (the effective
 * dedt). trace (nullable) receives before_kick, acceleration and the
 * post-kick conserved state (hydro.py:135-142). */
jx_status jx_force_kick(const jx_desc* d, const jx_forcing* f, void* U, jx_clock* clock,
                        const jx_trace* trace, void* workspace, size_t workspace_bytes,
                        jx_stream s);

/* One full evolve_isothermal cycle (run.py:40-61) with the state kept in S:
 * jx_begin_step, optional render, all stages (S -> A -> B ...), optional kick.
 * A and B are scratch states of S's shape. forcing may be NULL. No SGS hook
 * (callers with a hook drive jx_stage themselves). */
jx_status jx_step(const jx_desc* d, void* S, void* A, void* B, const jx_forcing* forcing,
                  jx_clock* clock, void* workspace, size_t workspace_bytes, jx_stream s);

/* One solve of a batch: the arguments of jx_step. forcing.raw_force == NULL
 * means unforced. */
typedef struct {
  jx_desc desc;
  void *S, *A, *B;
  jx_clock* clock;
  jx_forcing forcing;
  void* workspace;
  size_t workspace_bytes;
} jx_solve;

/* Batches advance many independent solves together (the reference evolves
 * one grid per evolve_isothermal call, run.py:20-69): per RK stage one
 * persistent launch per (precision, reconstruction, Riemann solver, kernel)
 * group walks a tile work list spanning all the group's grids. Solves must
 * have 3 or 4 variables (16-byte aligned states for 4). Each solve's
 * desc.tile_x/tile_y select its tile as in jx_step, restricted to the two
 * 3/4-variable kernels: 32 x h shared-memory tiles or 58 x h marching tiles
 * (0, 0 = the default of jx_tile_info). Results are bitwise the same as
 * running each solve alone with jx_step and the same descriptor.
 * jx_batch_plan writes a plan into host memory; copy it unchanged to device
 * memory of the same size and pass both to jx_batch_step, which enqueues one
 * evolve cycle of every solve (batched begin-step, renders, stages, kicks).
 * blocks_per_sm <= 0 picks the occupancy limit. */
jx_status jx_batch_plan_bytes(const jx_solve* solves, int32_t n, size_t* bytes);
jx_status jx_batch_plan(const jx_solve* solves, int32_t n, void* plan, size_t bytes);
jx_status jx_batch_step(const void* plan, const void* plan_dev, int32_t blocks_per_sm, jx_stream s);
/* Number of launch groups in a plan (-1 if not a plan). */
int32_t jx_batch_groups(const void* plan);

/* rk_stage (hydro.py:39-51) on whole arrays: U_out = combine(U, V, div),
 * V_out = V + delta*U when has_delta. n = number of elements. */
jx_status jx_rk_stage(int32_t dtype, int64_t n, const void* U, const void* V, const void* div,
                      double dt, double gam0, double gam1, double beta, double delta,
                      int32_t has_delta, void* U_out, void* V_out, jx_stream s);

/* flux_divergence (fluxes.py:283-287): (ny, nx, nv) face fluxes -> div. */
jx_status jx_flux_divergence(int32_t dtype, int32_t ny, int32_t nx, int32_t nv,
                             const void* flux_x, const void* flux_y, double dx, double dy,
                             void* div, jx_stream s);

/* stress_face_fluxes (fluxes.py:269-280): (ny, nx, 3) cell stress -> two
 * (ny, nx, 2) face momentum fluxes. */
jx_status jx_stress_face_fluxes(int32_t dtype, int32_t ny, int32_t nx, const void* tau,
                                void* flux_x, void* flux_y, jx_stream s);

/* Face-level operators (fluxes.py), for callers that use them directly; the
 * fused stage does not call them.
 * reconstruct_faces (fluxes.py:126-131) along axis (1 = x, 0 = y): left and
 * right primitive states (ny, nx, nv) at the low face of every cell, with the
 * ppmx/wenoz face density floor. */
jx_status jx_face_states(int32_t dtype, int32_t recon, int32_t ny, int32_t nx, int32_t nv,
                         const void* W, int32_t axis, double dfloor, void* left, void* right,
                         jx_stream s);
/* isothermal_flux (fluxes.py:207-219): gas + upwinded scalar fluxes of nface
 * faces (nface x nv arrays) in x/y component order. */
jx_status jx_face_flux(int32_t dtype, int32_t rsolver, int64_t nface, int32_t nv, int32_t axis,
                       const void* left, const void* right, double cs, void* flux, jx_stream s);
/* viscous_momentum_flux (fluxes.py:248-266): (ny, nx, 2) negative viscous
 * stress at the low faces along axis, from primitives W (ny, nx, nv). */
jx_status jx_viscous_flux(int32_t dtype, int32_t ny, int32_t nx, int32_t nv, const void* W,
                          double dx, double dy, double viscosity, double smagorinsky_cs,
                          int32_t axis, void* out, jx_stream s);

/* face_velocity_gradients (fluxes.py:227-238): dv_dx and dv_dy, each
 * (ny, nx, 2) = both velocity components, at the low faces along axis
 * (1 = x, 0 = y), from primitives W (ny, nx, nv). */
jx_status jx_face_velocity_gradients(int32_t dtype, int32_t ny, int32_t nx, int32_t nv, const void* W, double dx,
                                     double dy, int32_t axis, void* dv_dx, void* dv_dy, jx_stream s);
/* smagorinsky_viscosity (fluxes.py:241-245): Cs^2 dx dy sqrt(2 S:S) per
 * face from the gradients above; out has ncell values. */
jx_status jx_smagorinsky_viscosity(int32_t dtype, int64_t ncell, const void* dv_dx, const void* dv_dy, double dx,
                                   double dy, double smagorinsky_cs, void* out, jx_stream s);

/* Sum of (rho, rho*vx, rho*vy, ...) over the grid in float64 (the
 * box-integrated conservation check of run.py:186-187). out: nvar doubles. */
jx_status jx_box_sums(const jx_desc* d, const void* U, double* out, void* workspace,
                      size_t workspace_bytes, jx_stream s);

/* Tile shape and shared memory the stage kernel will use for `d`
 * (smem_bytes = 0 for marching tiles, which use registers and shuffles). */
jx_status jx_tile_info(const jx_desc* d, int32_t* tile_x, int32_t* tile_y, int64_t* smem_bytes);

/* modal_coefficients (forcing.py:63-100) on the host: the OU table
 * [updates][n_modes][2 dir][2 re/im] for the seed, bit-identical to the
 * reference's Python generator. modes: n_modes x 2 integers (kx, ky).
 * Returns 0, or -1 for null/negative arguments. Host memory only. */
int32_t jx_ou_table(const int32_t* modes, int32_t n_modes, double Lx, double Ly, int32_t nlow,
                    int32_t nhigh, double npeak, double sol_fraction, int64_t seed, double tcorr,
                    double dt_update, int32_t updates, double* out);

/* Peak probe: `blocks` x 256 threads each run `chains` (8, 16 or 32)
 * independent chains of `iters` dependent FMAs in the given dtype
 * (2*chains*iters flops per thread). Timed by the caller with events to
 * measure the FP64/FP32 pipe rate. sink (device, >= blocks doubles) is never
 * written in practice. No counterpart in the reference. */
jx_status jx_probe_fma(int32_t dtype, int32_t blocks, int32_t iters, int32_t chains, double* sink,
                       jx_stream s);

/* Arithmetic probe for tests: for i < n, rcp_out[i] = 1/b[i],
 * div_out[i] = a[i]/b[i] (the quotient of the limiter and HLLE weights)
 * and geo_out[i] = sqrt(|a[i]|) sqrt(|b[i]|) as the stage kernels compute
 * them in `dtype` (device arrays of that type). */
jx_status jx_probe_math(int32_t dtype, int64_t n, const void* a, const void* b, void* rcp_out,
                        void* div_out, void* geo_out, jx_stream s);

#ifdef __cplusplus
}
#endif
#endif /* JX_H */
