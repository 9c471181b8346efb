/*
 * wb_capi.h -- C ABI of the GB300-native well-balanced Euler-with-gravity step.
 *
 * Drop-in boundary for the step routines of hanveiga/fvm-source-wb.  The reference
 * binds them as Fortran external subroutines with implicit interfaces and sizes taken
 * from module parameters; a Fortran driver reaches this library through an
 * ISO_C_BINDING interface module (bind(C, name="wb_...")) declared against this header.
 *
 * Conventions
 *   - every entry point returns an int status: WB_OK (0) or a negative WB_ERR_* code;
 *     wb_last_error(ctx) gives the message of the last failure on that context;
 *   - host arrays are caller-owned and only read/written during the call;
 *   - device buffers are owned by the context; one CUDA stream per context; a context
 *     is used by one host thread at a time;
 *   - modal state layout WB_LAYOUT_SOA:        delta[(v*nb + m)*ny*nx + j*nx + i]
 *                  layout WB_LAYOUT_FORTRAN:    u(nvar, nx, ny, k+1, k+1) column-major,
 *                  the reference's array layout (tensor basis WB_BASIS_Q only);
 *     v = 0..3 is (rho, rho*u, rho*v, E) of the PERTURBATION about the equilibrium;
 *     mode m <-> degrees (a, b) as listed by wb_mode_list.
 */
#ifndef WB_CAPI_H
#define WB_CAPI_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WB_OK 0
#define WB_ERR_CONFIG (-1)      /* invalid configuration */
#define WB_ERR_CUDA (-2)        /* CUDA runtime failure (message keeps cudaGetErrorString) */
#define WB_ERR_NONPHYSICAL (-3) /* device flag: non-finite or non-positive rho/p in a cell mean */
#define WB_ERR_TIMEOUT (-4)     /* a bounded device wait gave up */
#define WB_ERR_ARG (-5)         /* bad argument (null pointer, bad layout, size out of range) */
#define WB_ERR_NOMEM (-6)       /* device allocation failed */
#define WB_ERR_STATE (-7)       /* call not valid in the context's current state */

/* enumerations */
#define WB_BASIS_Q 0        /* tensor Legendre Q_k, (k+1)^2 modes (2d/benchmark_2d_dg.f90) */
#define WB_BASIS_P 1        /* total-degree P_k, (k+1)(k+2)/2 modes */
#define WB_BC_PERIODIC 0    /* bc=1 of 2d/parameters_dg_2d.f90 */
#define WB_BC_COPY 1        /* bc=2,3: ghost = copy of the edge cell's perturbation */
#define WB_EQ_NONE 0        /* zero equilibrium (nequilibrium=3) */
#define WB_EQ_ISOTHERMAL 1  /* rho = rho0 exp(-(rho0/p0) Phi), p = p0 exp(-(rho0/p0) Phi) */
#define WB_EQ_POLYTROPE 2   /* p = K rho^gamma, rho = (1 - (gamma-1)/(gamma K) Phi)^(1/(gamma-1)) */
#define WB_LLF_MAXABS 0     /* lambda = max(|v_n|+c) over both sides */
#define WB_LLF_REF2D 1      /* lambda = max(|v_n+c|) as compute_llflux of 2d/benchmark_2d_dg.f90 */
#define WB_PREC_FP64 0      /* "plain": FP64 state, literal F(u_eq+d) - F(u_eq) split */
#define WB_PREC_FP32 1      /* FP64 equilibrium tables + FP32 perturbation, exact-difference fluxes */
#define WB_RIEMANN_LLF 0    /* compute_llflux (2d/benchmark_2d_dg.f90:968-988); riemann=1 */
#define WB_RIEMANN_HLLC 1   /* riemann_hllc (dg_with_source.f90:1318-1374); riemann=2 */
#define WB_LIMITER_NONE 0
#define WB_LIMITER_MINMOD 1     /* limiter_type '1OR' (compute_limiter) on the perturbation */
#define WB_LIMITER_POSITIVITY 2 /* limiter_type 'ONP' (compute_positivity) in delta form */
#define WB_RK2 0            /* SSP-RK2 ('EQL' branch of evolve) */
#define WB_RK54 1           /* SSP-RK(5,4) ('RK4' branch of evolve) */
#define WB_LAYOUT_SOA 0
#define WB_LAYOUT_FORTRAN 1

typedef struct {
  int32_t nx, ny;        /* cells per direction (>= 1) */
  int32_t order;         /* polynomial degree k, 0..2 */
  int32_t basis;         /* WB_BASIS_* */
  int32_t bc_x, bc_y;    /* WB_BC_* */
  int32_t eq_kind;       /* WB_EQ_* */
  int32_t llf_speed;     /* WB_LLF_* */
  int32_t limiter;       /* WB_LIMITER_*: 0 off, 1 minmod moment limiter on the perturbation
                            (compute_limiter, 2d/limiters.f90:203-309), 2 Zhang-Shu
                            positivity limiter (compute_positivity, :478-654) in delta form */
  int32_t precision;     /* WB_PREC_* */
  int32_t integrator;    /* WB_RK2 or WB_RK54 */
  int32_t tile_x, tile_y;/* CTA tile in cells; 0 = the tuned shape from the tile cache,
                            else FP32 32x16 at two cells per thread for degrees 0 and 1
                            (total-degree basis), 32x8 otherwise; FP64 16x8 */
  int32_t device;        /* CUDA device ordinal */
  int32_t riemann;       /* WB_RIEMANN_LLF or WB_RIEMANN_HLLC */
  int32_t cells_per_thread; /* cells each thread of the tile computes (the CTA has
                            tile_x * tile_y / cells_per_thread threads); 0 = 1, or the
                            tuned default when tile_x is 0 */
  double gamma;
  double gx, gy;         /* Phi = gx x + gy y */
  double rho0, p0;       /* isothermal reference state */
  double kpoly;          /* polytropic constant K */
  double lx, ly;         /* domain [0,lx] x [0,ly] */
  double lim_norm;       /* minmod slope scaling (reference: 3) */
  double lim_M;          /* TVB constant M (slopes with |norm s| < M h^2 untouched) */
  double lim_tol;        /* re-limit a cell only if a slope changes by more than this */
  double cfl;            /* CFL number */
  double pos_eps;        /* positivity floor of density and pressure (reference eps 1e-10) */
} wb_config;

/* seeded perturbation generator (initial condition), evaluated on the device in FP64 */
typedef struct {
  int32_t kind;          /* 0 zero, 1 Gaussian pressure bump, 2 multimode velocity */
  int32_t nmodes;        /* kind 2: Fourier modes (<= 32) */
  double amp;
  double xc, yc, sigma;  /* kind 1 */
  double kx[32], ky[32], phase_u[32], phase_v[32], weight[32]; /* kind 2 */
} wb_perturbation;

typedef struct wb_ctx wb_ctx;

/* --- configuration and lifetime ------------------------------------------------ */
/* Fills the reference's defaults (2d/parameters_dg_2d.f90:1-40 where they apply). */
int wb_config_default(wb_config *cfg);
/* Creates a context: validates cfg, allocates the state and equilibrium tables on
 * cfg->device.  Replaces the module-parameter setup of 2d/parameters_dg_2d.f90 and
 * get_coords/get_equilibrium_solution (2d/benchmark_2d_dg.f90:93-120,594-622). */
int wb_create(const wb_config *cfg, wb_ctx **out);
int wb_destroy(wb_ctx *ctx);
const char *wb_last_error(const wb_ctx *ctx);
/* Replaces the context's hydrostatic equilibrium (get_equilibrium_solution,
 * 2d/benchmark_2d_dg.f90:594-622): kind WB_EQ_*, Phi = gx x + gy y, params = {rho0, p0,
 * kpoly} (null keeps them).  Validated like wb_create; the perturbation state is kept (it
 * is now a perturbation of the new equilibrium); waits for the context's work first. */
int wb_set_equilibrium(wb_ctx *ctx, int32_t kind, double gx, double gy, const double *params);
const char *wb_status_string(int status);
/* number of modes per variable; the (a,b) degree list in the library's order */
int wb_num_modes(int order, int basis);
int wb_mode_list(int order, int basis, int32_t *deg_x, int32_t *deg_y);

/* --- state transfer ------------------------------------------------------------ */
/* Upload / download the perturbation modes (FP64 host arrays).  Download returns the
 * limited state, i.e. what apply_limiter would leave after the last stage. */
int wb_upload_state(wb_ctx *ctx, const double *delta, int32_t layout);
int wb_download_state(wb_ctx *ctx, double *delta, int32_t layout);
/* same with FP32 host arrays (SoA only) */
int wb_upload_state_f32(wb_ctx *ctx, const float *delta);
int wb_download_state_f32(wb_ctx *ctx, float *delta);
/* Pipelined host I/O (FP32 contexts): enqueues the upload of `in` as the state, `nsteps`
 * steps (dt > 0 fixed, else CFL) and the download of the limited result into `out`, and
 * returns at once.  Successive calls overlap: the upload of call k+1 and the download of
 * call k-1 run on their own streams while call k steps (ping-pong device staging).
 * `in` and `out` (dense SoA float arrays, page-locked for the copies to be asynchronous)
 * belong to the library until wb_sync.  Time and step counter continue across calls.
 * (No reference routine: the host-to-device pipeline of a drop-in driver.) */
int wb_step_io_f32(wb_ctx *ctx, const float *in, float *out, int32_t nsteps, double dt);
/* Failure-detection self-test: runs the bounded device wait of the tile staging (the
 * mbarrier wait of the TMA copies) on a barrier that nothing completes, limited to
 * `polls` polls.  Returns WB_ERR_TIMEOUT (the expected result: the wait gave up and
 * reported it through the context's error word), then clears the word so the context
 * stays usable. */
int wb_selftest_wait_timeout(wb_ctx *ctx, int32_t polls);
/* The resident state exactly as stored (SoA; double for FP64 contexts, float for FP32),
 * before the limit-on-load: what a checkpoint needs so that a restart through
 * wb_upload_state / wb_upload_state_f32 continues bit for bit.  (No reference routine:
 * the reference keeps its state in memory.) */
int wb_download_state_raw(wb_ctx *ctx, void *delta);
/* Projects a seeded perturbation onto the modes on the device (the IC + projection of
 * get_initial_conditions/get_modes_from_nodes, 2d/benchmark_2d_dg.f90:122-153,497-542);
 * resets t and the step counter. */
int wb_init_perturbation(wb_ctx *ctx, const wb_perturbation *ic);
/* Device address of the resident state (SoA, element type per precision) and the
 * element stride between (variable, mode) planes. */
int wb_device_state(wb_ctx *ctx, void **dptr, size_t *plane_stride);

/* --- the step routines ------------------------------------------------------- */
/* dudt = L(delta) for host arrays: drop-in for compute_update(delta_u, x, y, u_eq, dudt),
 * 2d/benchmark_2d_dg.f90:1137-1479 (x, y, u_eq are implied by the context), in the
 * well-balanced split of compute_update_exact_delta, dg_with_source.f90:1749-2031.
 * The input is not limited (compute_update does not limit). */
int wb_compute_update(wb_ctx *ctx, const double *delta_u, double *dudt, int32_t layout);
/* Limits the resident state in place: apply_limiter(u), 2d/benchmark_2d_dg.f90:1516-1555,
 * with compute_limiter (2d/limiters.f90:203-309) or compute_positivity (:478-654) as
 * cfg.limiter selects, applied to the perturbation. */
int wb_apply_limiter(wb_ctx *ctx);
/* Directional maximum wave speeds max(|u|+c), max(|v|+c) over cell means of the full
 * state: compute_max_speed(u, cs_max, v_xmax, v_ymax, speed_max), :826-870. */
int wb_max_speed(wb_ctx *ctx, double *smax_x, double *smax_y);
/* Advances nsteps time steps with cfg->integrator (the stage loop of evolve,
 * 2d/benchmark_2d_dg.f90:666-747).  dt > 0: fixed step; dt <= 0: CFL step computed
 * on the device every step from the fused wave-speed reduction.  Asynchronous on the
 * context stream; errors from the device flag surface at the next synchronising call. */
int wb_step(wb_ctx *ctx, int32_t nsteps, double dt);
/* Runs until t >= tend (or max_steps) with CFL steps clipped at tend: evolve,
 * 2d/benchmark_2d_dg.f90:624-775.  Synchronising. */
int wb_evolve(wb_ctx *ctx, double tend, int32_t max_steps, int32_t *steps_done, double *t_out);
/* Waits for the context stream; reports a device-side non-physical flag. */
int wb_sync(wb_ctx *ctx);  /* also completes wb_step_io_f32 copies */
int wb_get_time(wb_ctx *ctx, double *t, int64_t *steps);
/* Sets the simulated time and step counter (checkpoint restart; the reference keeps t
 * in evolve's locals and has no restart). */
int wb_set_time(wb_ctx *ctx, double t, int64_t steps);

/* Autotuner: times every compiled tile shape (CTA tile of cells, and cells per thread) for
 * this context's precision, degree, basis and grid over `steps` steps of the current state
 * (restored afterwards), keeps the fastest and records it in the tile cache (the file named
 * by the environment variable WB_TILE_CACHE, else tile_cache.txt beside the library), which
 * wb_create consults when cfg->tile_x == 0.  Compiled shapes: FP32 32x8 and 16x16 at one
 * cell per thread, 32x16 at two (total-degree basis and degree 0), 32x32 at four (degree
 * 0); FP64 16x8 and 16x4.  The tiled loop is the per-cell work of compute_update,
 * 2d/benchmark_2d_dg.f90:1207-1244.  No counterpart in the reference. */
int wb_autotune(wb_ctx *ctx, int32_t steps, int32_t *tile_x, int32_t *tile_y,
                int32_t *cells_per_thread);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own work
 * against it or time it with CUDA events.  No counterpart in the reference (serial). */
int wb_get_stream(wb_ctx *ctx, void **stream);
/* When on, every stage-kernel launch is bracketed by CUDA events on the context stream;
 * wb_stage_stats returns the summed kernel time and launch count since the last call
 * (and resets them).  No counterpart in the reference (it has no timers). */
int wb_profile_stages(wb_ctx *ctx, int32_t on);
int wb_stage_stats(wb_ctx *ctx, double *total_ms, int64_t *launches);

/* --- diagnostics ---------------------------------------------------------------- */
/* Error norms of the (limited) resident state against another context's state on the
 * same grid and basis (other may be NULL: norms of the state itself), in FP64:
 * compute_error, 2d/benchmark_2d_dg.f90:23-89 (L1, Linf, L2 per conserved variable). */
int wb_norms(wb_ctx *ctx, wb_ctx *other, double l1[4], double linf[4], double l2[4]);
/* FP64 domain integrals of the full conserved state (equilibrium + perturbation). */
int wb_conserved_sums(wb_ctx *ctx, double sums[4]);

/* Error norms (L1, Linf, L2 per conserved variable, as wb_norms) of two device-resident
 * FP64 modal states a and b (SoA, plane_stride elements between (variable, mode) planes,
 * the same stride and [variable][mode][plane] layout for both -- wb_device_state gives a
 * context's; b may be NULL for the norms of a) that allocates no device memory.  No counterpart in
 * the reference.  It is for callers that cannot call cudaMalloc where they need the norms:
 * a host whose device memory is all owned by its own pool or by another runtime, or a time
 * loop that must not take the device-wide synchronisation cudaMalloc/cudaFree imply.
 * Its reduction scratch is a fixed array inside the library, 1.5 MB on every device that
 * loads the library and held until the process exits, so grids are limited to
 * WB_NORMS_NOALLOC_MAX_CELLS cells, and a grid whose 32x8-cell blocks outnumber the
 * array's 16,384 partial slots (a narrow grid such as 33 x 127,000) returns WB_ERR_ARG too
 * (use wb_norms).  The first call on a device sets that device up (looks up the array's
 * device address and uploads the basis tables).  Every call copies its results back and
 * waits for `stream`, so no call may be made while that stream is being captured into a
 * graph: such a call returns WB_ERR_ARG and leaves the capture as it was.  The set-up
 * belongs to the device's CUDA context: after that context is torn
 * down (cudaDeviceReset) and created again, the next call sets the device up again.  Every call
 * uses the same array, so calls that overlap on the GPU (other streams, other threads)
 * race.  stream may be NULL (the default stream); the call waits for it before it returns
 * the host results. */
#define WB_NORMS_NOALLOC_MAX_CELLS 4194304
int wb_norms_device_noalloc(int32_t nx, int32_t ny, int32_t order, int32_t basis, double lx,
                            double ly, const double *a, const double *b, size_t plane_stride,
                            void *stream, double l1[4], double linf[4], double l2[4]);
/* Text snapshot in the reference's format: output_file, 2d/benchmark_2d_dg.f90:468-495 --
 * one line per cell (x index outer, y inner) with x, y of the cell's first Gauss point
 * and the primitive perturbation w - w_eq there for variables var..4, each written as
 * Fortran 1PE12.5, separated by one blank (the format's 1X; no blank ends a record, as
 * Fortran writes it). */
int wb_write_dat(wb_ctx *ctx, const char *path, int32_t var);
/* Reads a text snapshot written in that format ('(7(1PE12.5,1X))', one record per line,
 * a record of more than 7 values continued on the next lines, 7 per line) into
 * values[row * ncols + col]; *nrows receives the records read.  Accepts the E-less
 * three-digit exponent form (1.23456-100).  WB_ERR_ARG for a missing file, a token that
 * is not a number, a record of another length, or more than `capacity` records.  The
 * reference reads its snapshots with np.loadtxt in get_image (post_processing2d.py:55-64):
 * columns x, y, then the fields, reshaped to (nx, ny) with y fastest.  Host only. */
int wb_read_dat(const char *path, int32_t ncols, double *values, int64_t capacity, int64_t *nrows);

/* --- batched form -------------------------------------------------------------- */
typedef struct wb_batch wb_batch;
/* n independent instances (each its own grid, order, equilibrium, limiter), total-degree
 * basis, FP32-perturbation form, SSP-RK2, advanced together: per step one launch that
 * computes every instance's time step, then per RK stage one persistent launch per group
 * (instances of one degree on one tile shape) over a work list of cell tiles, each group on
 * its own branch of a CUDA graph that replays the step sequence.  An instance's tile_x/tile_y/cells_per_thread pin
 * its tile (32x8 or 16x16 at one cell per thread, 32x16 at two, 32x32 at four for degree
 * 0); 0 leaves it to the batch (until wb_batch_autotune: 32x16 at two cells per thread for
 * degrees 0 and 1, 32x8 for degree 2). */
int wb_batch_create(const wb_config *cfgs, int32_t n, wb_batch **out);
int wb_batch_destroy(wb_batch *b);
const char *wb_batch_last_error(const wb_batch *b);
int wb_batch_init_perturbation(wb_batch *b, const wb_perturbation *ics);
/* nsteps steps; each instance takes its own CFL dt (dt <= 0) or the fixed dt */
int wb_batch_step(wb_batch *b, int32_t nsteps, double dt);
/* Waits for the batch's work and checks every instance's device error word (one copy for
 * the whole batch): WB_ERR_NONPHYSICAL or WB_ERR_TIMEOUT, with the first failing instance
 * named in wb_batch_last_error. */
int wb_batch_sync(wb_batch *b);
/* Tile autotuner of the batched form: for every (degree, size class) group of instances
 * without a pinned tile -- size class 0: max(nx, ny) < 128, 1: the rest -- times `reps`
 * stage launches of each compiled tile shape and cells per thread of that degree on those
 * instances and keeps the fastest.  The instances' states are not changed.  tiles
 * (optional, int32[18]) receives the choice (TX, TY, cells per thread) for degree K and
 * class s at [(2K + s) * 3]. */
int wb_batch_autotune(wb_batch *b, int32_t reps, int32_t *tiles);
int wb_batch_download(wb_batch *b, int32_t index, double *delta);
int wb_batch_total_dofs(wb_batch *b, int64_t *dofs);

/* --- 1D well-balanced finite volume (the fvm.f90 / benchmark_1d.f90 path) --------- */
typedef struct wb1d_ctx wb1d_ctx;
typedef struct {
  int32_t nx;
  int32_t bc;            /* WB_BC_PERIODIC or WB_BC_COPY (equilibrium-extrapolated) */
  int32_t limiter;       /* 0 first order, 1 minmod MUSCL on the perturbation */
  int32_t eq_kind;       /* WB_EQ_ISOTHERMAL or WB_EQ_POLYTROPE */
  int32_t device;
  int32_t scheme;        /* WB1D_EQL or WB1D_WB1 */
  double gamma, g, rho0, p0, kpoly, lx, cfl;
} wb1d_config;
#define WB1D_EQL 0  /* compute_update 'EQL' (benchmark_1d.f90:263-377): equilibrium + delta faces */
#define WB1D_WB1 1  /* compute_update_sr 'WB1' (benchmark_1d.f90:553-747): hydrostatic reconstruction */
/* compute_update ('EQL' or 'WB1') + evolve of benchmark_1d.f90:200-377 on the device */
int wb1d_create(const wb1d_config *cfg, wb1d_ctx **out);
int wb1d_destroy(wb1d_ctx *c);
const char *wb1d_last_error(const wb1d_ctx *c);
int wb1d_upload(wb1d_ctx *c, const double *delta);      /* delta[i*3 + v] */
int wb1d_download(wb1d_ctx *c, double *delta);
int wb1d_compute_update(wb1d_ctx *c, const double *delta, double *dudt);
int wb1d_evolve(wb1d_ctx *c, double tend, int32_t max_steps, int32_t *steps_done, double *t_out);
/* Text snapshot of the 1D state: output_file, benchmark_1d.f90:69-100 -- one line per cell
 * with the cell centre x and the primitive perturbation w - w_eq at the centre for
 * variables var..3 of (rho, u, p) (the reference writes var = 3), each as 1PE12.5,
 * separated by one blank; read back with wb_read_dat. */
int wb1d_write_dat(wb1d_ctx *c, const char *path, int32_t var);

#ifdef __cplusplus
}
#endif
#endif
