// wb_capi.cu -- host implementation of the C ABI in include/wb_capi.h for the 2D
// well-balanced step: context lifetime, state transfer, the stage loop of evolve, and
// diagnostics.  Kernels live in the per-precision translation units.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wb_capi.h"
#include "wb_internal.h"
#include "wb_tables.h"

using namespace wb;

struct wb_ctx {
  wb_config cfg;
  int nb = 0, nq = 0, nbuf = 0;
  long long ncell = 0, plane = 0;  // cells (nx * ny); elements between (var, mode) planes
  int pitch = 0;                     // elements between rows of a plane: nx, or nx rounded up
                                     // to 16 bytes for batch instances
  size_t esize = 0, state_bytes = 0;
  void *buf[6] = {nullptr};
  int cur = 0;
  double *scratch64 = nullptr;  // FP64 state-sized staging (lazy)
  void *fxv = nullptr, *fxf = nullptr, *fyv = nullptr, *fyf = nullptr;  // kernel-precision
  double *fxv64 = nullptr, *fxf64 = nullptr, *fyv64 = nullptr, *fyf64 = nullptr;
  Tab1D<double> *Td = nullptr;  // device copy of the FP64 1D tables
  DevState *dev = nullptr;
  double *partial = nullptr, *diag_out = nullptr;
  cudaStream_t stream = nullptr;
  int parity = 0;
  bool speed_valid = false;
  int TX = 32, TY = 8, CPT = 1;  // stage tile and cells per thread
  std::string err;
  bool profile = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;  // recorded stage launches
  std::vector<cudaEvent_t> ev_pool;
  // TMA descriptors of the state buffers, per staged tile shape (built on first use)
  struct Tmap {
    const void *base;
    int tx, ty;
    bool ok;
    CUtensorMap map;
  };
  std::deque<Tmap> tmaps;  // stable addresses
  // pipelined host I/O (wb_step_io_f32): copy streams, ping-pong device staging, events
  bool io_init = false;
  int io_k = 0;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  void *io_in[2] = {nullptr, nullptr}, *io_out[2] = {nullptr, nullptr};
  cudaEvent_t in_ready[2] = {}, in_free[2] = {}, out_ready[2] = {}, out_free[2] = {};
};

namespace {

int set_err(wb_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}
#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return set_err(ctx, WB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

bool is_fp32(const wb_ctx *c) { return c->cfg.precision == WB_PREC_FP32; }

int validate(const wb_config *c, std::string &why) {
  if (c->nx < 1 || c->ny < 1) return why = "nx, ny must be >= 1", WB_ERR_CONFIG;
  if ((long long)c->nx * c->ny > (1LL << 31) - 1) return why = "nx*ny too large", WB_ERR_CONFIG;
  if (c->order < 0 || c->order > KMAX) return why = "order must be 0..2", WB_ERR_CONFIG;
  if (c->basis != WB_BASIS_Q && c->basis != WB_BASIS_P) return why = "bad basis", WB_ERR_CONFIG;
  if ((c->bc_x != 0 && c->bc_x != 1) || (c->bc_y != 0 && c->bc_y != 1))
    return why = "bad boundary condition", WB_ERR_CONFIG;
  if (c->eq_kind < 0 || c->eq_kind > 2) return why = "bad eq_kind", WB_ERR_CONFIG;
  if (c->llf_speed != 0 && c->llf_speed != 1) return why = "bad llf_speed", WB_ERR_CONFIG;
  if (c->precision != WB_PREC_FP64 && c->precision != WB_PREC_FP32)
    return why = "bad precision", WB_ERR_CONFIG;
  if (c->integrator != WB_RK2 && c->integrator != WB_RK54) return why = "bad integrator", WB_ERR_CONFIG;
  if (!(c->gamma > 1.0)) return why = "gamma must be > 1", WB_ERR_CONFIG;
  if (!(c->lx > 0.0) || !(c->ly > 0.0)) return why = "domain lengths must be > 0", WB_ERR_CONFIG;
  if (!(c->cfl > 0.0)) return why = "cfl must be > 0", WB_ERR_CONFIG;
  if (c->eq_kind == WB_EQ_ISOTHERMAL && !(c->rho0 > 0.0 && c->p0 > 0.0))
    return why = "isothermal rho0, p0 must be > 0", WB_ERR_CONFIG;
  if (c->eq_kind == WB_EQ_POLYTROPE) {
    if (!(c->kpoly > 0.0)) return why = "kpoly must be > 0", WB_ERR_CONFIG;
    double k = (c->gamma - 1.0) / (c->gamma * c->kpoly);
    double phimax = std::fmax(0.0, c->gx * c->lx) + std::fmax(0.0, c->gy * c->ly);
    if (!(1.0 - k * phimax > 0.0)) return why = "polytrope density vanishes inside the domain", WB_ERR_CONFIG;
  }
  if (c->riemann != WB_RIEMANN_LLF && c->riemann != WB_RIEMANN_HLLC)
    return why = "bad riemann (0 LLF, 1 HLLC)", WB_ERR_CONFIG;
  if (c->limiter < 0 || c->limiter > 2) return why = "bad limiter (0 off, 1 minmod, 2 positivity)", WB_ERR_CONFIG;
  if (c->limiter == 1 && !(c->lim_norm > 0.0)) return why = "lim_norm must be > 0", WB_ERR_CONFIG;
  if (c->limiter == 2 && !(c->pos_eps > 0.0)) return why = "pos_eps must be > 0", WB_ERR_CONFIG;
  if (c->tile_x < 0 || c->tile_y < 0 || c->cells_per_thread < 0) return why = "bad tile", WB_ERR_CONFIG;
  if (c->cells_per_thread > 0 && c->tile_x == 0)
    return why = "cells_per_thread needs a tile (tile_x, tile_y)", WB_ERR_CONFIG;
  if (c->tile_x > 0 || c->tile_y > 0) {
    const int cpt = c->cells_per_thread > 0 ? c->cells_per_thread : 1;
    if (!tile_supported(c->precision == WB_PREC_FP32, c->order, c->basis, c->tile_x, c->tile_y, cpt))
      return why = "tile shape not compiled (FP32: 32x8, 16x16, 32x16 at 2 cells per thread, "
                   "degree 0 also 32x32 at 4; FP64: 16x8, 16x4)", WB_ERR_CONFIG;
  }
  return WB_OK;
}

template <typename R>
StageArgs<R> base_args(const wb_ctx *c) {
  StageArgs<R> A;
  std::memset(&A, 0, sizeof(A));
  const wb_config &g = c->cfg;
  A.nx = g.nx;
  A.ny = g.ny;
  A.pitch = c->pitch;
  A.plane = c->plane;
  A.bc_x = g.bc_x;
  A.bc_y = g.bc_y;
  A.llf_speed = g.llf_speed;
  A.limiter = g.limiter;
  A.lim_y = 1;
  A.riemann = g.riemann;
  A.eq_kind = g.eq_kind;
  double dx = g.lx / g.nx, dy = g.ly / g.ny;
  A.dx = (R)dx;
  A.dy = (R)dy;
  A.hidx = (R)(0.5 / dx);
  A.hidy = (R)(0.5 / dy);
  A.gamma = (R)g.gamma;
  A.gm1 = (R)(g.gamma - 1.0);
  A.igm1 = (R)(1.0 / (g.gamma - 1.0));
  A.hgam = (R)(g.gamma / (g.gamma - 1.0));
  A.gx = (R)g.gx;
  A.gy = (R)g.gy;
  A.rho0 = (R)g.rho0;
  A.p0 = (R)g.p0;
  A.kpoly = (R)g.kpoly;
  A.npoly = (R)(1.0 / (g.gamma - 1.0));
  A.lim_norm = (R)g.lim_norm;
  A.lim_inorm = (R)(1.0 / g.lim_norm);
  A.lim_Mdx2 = (R)(g.lim_M * dx * dx);
  A.lim_Mdy2 = (R)(g.lim_M * dy * dy);
  A.lim_tol = (R)g.lim_tol;
  A.pos_eps = (R)g.pos_eps;
  A.fxv = (const R *)c->fxv;
  A.fxf = (const R *)c->fxf;
  A.fyv = (const R *)c->fyv;
  A.fyf = (const R *)c->fyf;
  A.dt_mode = 0;
  A.parity = c->parity;
  A.cfl_over = g.cfl / (2.0 * g.order + 1.0);
  A.tend = -1.0;
  A.ddx = dx;
  A.ddy = dy;
  A.dev = c->dev;
  return A;
}

AuxArgs aux_args(const wb_ctx *c) {
  AuxArgs A;
  std::memset(&A, 0, sizeof(A));
  const wb_config &g = c->cfg;
  A.nx = g.nx;
  A.ny = g.ny;
  A.pitch = c->pitch;
  A.plane = c->plane;
  A.bc_x = g.bc_x;
  A.bc_y = g.bc_y;
  A.limiter = g.limiter;
  A.eq_kind = g.eq_kind;
  A.dx = g.lx / g.nx;
  A.dy = g.ly / g.ny;
  A.gamma = g.gamma;
  A.gx = g.gx;
  A.gy = g.gy;
  A.rho0 = g.rho0;
  A.p0 = g.p0;
  A.kpoly = g.kpoly;
  A.npoly = 1.0 / (g.gamma - 1.0);
  A.lim_norm = g.lim_norm;
  A.lim_Mdx2 = g.lim_M * A.dx * A.dx;
  A.lim_Mdy2 = g.lim_M * A.dy * A.dy;
  A.lim_tol = g.lim_tol;
  A.fxv = c->fxv64;
  A.fxf = c->fxf64;
  A.fyv = c->fyv64;
  A.fyf = c->fyf64;
  return A;
}

template <typename T>
int dalloc(wb_ctx *ctx, T **p, size_t bytes) {
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_err(ctx, WB_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(bytes) +
                                          " bytes): " + cudaGetErrorString(e));
  }
  return WB_OK;
}

// Copies the NV * nb planes of a state between a dense host array [plane][ny][nx] of
// elements of es bytes and a device buffer [plane stride][ny rows of pitch elements].
int copy_planes(wb_ctx *ctx, void *dst, const void *src, size_t es, cudaMemcpyKind kind,
                cudaStream_t st) {
  const int nrow = NV * ctx->nb;
  const bool to_dev = kind == cudaMemcpyHostToDevice;
  const size_t planeb = (size_t)ctx->plane * es, denseb = (size_t)ctx->ncell * es;
  if (ctx->pitch == ctx->cfg.nx && ctx->plane == ctx->ncell) {
    // planes without padding: the state is one contiguous block on both sides
    CK(cudaMemcpyAsync(dst, src, denseb * nrow, kind, st));
    return WB_OK;
  }
  if (ctx->pitch == ctx->cfg.nx) {  // one 2D copy: a plane is one row
    CK(cudaMemcpy2DAsync(dst, to_dev ? planeb : denseb, src, to_dev ? denseb : planeb, denseb, nrow,
                         kind, st));
    return WB_OK;
  }
  const size_t rowb = (size_t)ctx->cfg.nx * es, pitchb = (size_t)ctx->pitch * es;
  for (int r = 0; r < nrow; ++r) {
    char *d = (char *)dst + (size_t)r * (to_dev ? planeb : denseb);
    const char *q = (const char *)src + (size_t)r * (to_dev ? denseb : planeb);
    CK(cudaMemcpy2DAsync(d, to_dev ? pitchb : rowb, q, to_dev ? rowb : pitchb, rowb, ctx->cfg.ny,
                         kind, st));
  }
  return WB_OK;
}

int ensure_scratch(wb_ctx *ctx) {
  if (ctx->scratch64) return WB_OK;
  return dalloc(ctx, &ctx->scratch64, (size_t)NV * ctx->nb * ctx->plane * sizeof(double));
}

template <typename R>
int upload_table(wb_ctx *ctx, void **dst, const std::vector<double> &v) {
  std::vector<R> h(v.begin(), v.end());
  if (*dst == nullptr) {  // first build allocates; a rebuild overwrites in place
    int rc = dalloc(ctx, (R **)dst, h.size() * sizeof(R));
    if (rc) return rc;
  }
  CK(cudaMemcpy(*dst, h.data(), h.size() * sizeof(R), cudaMemcpyHostToDevice));
  return WB_OK;
}

// Equilibrium factor tables of ctx->cfg (FP64 copy, and the kernel-precision copy).
int build_eq_tables(wb_ctx *ctx, const double *xq) {
  const wb_config *cfg = &ctx->cfg;
  EqParams ep{cfg->eq_kind, cfg->gamma, cfg->gx, cfg->gy, cfg->rho0, cfg->p0, cfg->kpoly};
  std::vector<double> fxv, fxf, fyv, fyf;
  make_eq_tables(ep, cfg->nx, cfg->ny, cfg->lx, cfg->ly, ctx->nq, xq, fxv, fxf, fyv, fyf);
  int rc;
  if ((rc = upload_table<double>(ctx, (void **)&ctx->fxv64, fxv))) return rc;
  if ((rc = upload_table<double>(ctx, (void **)&ctx->fxf64, fxf))) return rc;
  if ((rc = upload_table<double>(ctx, (void **)&ctx->fyv64, fyv))) return rc;
  if ((rc = upload_table<double>(ctx, (void **)&ctx->fyf64, fyf))) return rc;
  if (is_fp32(ctx)) {
    if ((rc = upload_table<float>(ctx, &ctx->fxv, fxv))) return rc;
    if ((rc = upload_table<float>(ctx, &ctx->fxf, fxf))) return rc;
    if ((rc = upload_table<float>(ctx, &ctx->fyv, fyv))) return rc;
    if ((rc = upload_table<float>(ctx, &ctx->fyf, fyf))) return rc;
  } else {
    if ((rc = upload_table<double>(ctx, &ctx->fxv, fxv))) return rc;
    if ((rc = upload_table<double>(ctx, &ctx->fxf, fxf))) return rc;
    if ((rc = upload_table<double>(ctx, &ctx->fyv, fyv))) return rc;
    if ((rc = upload_table<double>(ctx, &ctx->fyf, fyf))) return rc;
  }
  return WB_OK;
}

void *state_buf(wb_ctx *c, int off) { return c->buf[(c->cur + off) % c->nbuf]; }

// cuTensorMapEncodeTiled, from the driver through the runtime (no link to libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// The tensor map that stages a (TX+8) x (TY+2) x planes block of state buffer `base`
// ([plane][ny][nx], plane stride `plane` elements) into the tile layout of wb_types.h;
// null where TMA cannot address it (rows not a multiple of 16 bytes) or it is disabled
// (environment WB_NO_TMA=1).
const CUtensorMap *state_tmap(wb_ctx *ctx, const void *base, int TX, int TY) {
  static const bool off = [] {
    const char *e = std::getenv("WB_NO_TMA");
    return e && *e && *e != '0';
  }();
  if (off) return nullptr;
  for (auto &m : ctx->tmaps)
    if (m.base == base && m.tx == TX && m.ty == TY) return m.ok ? &m.map : nullptr;
  wb_ctx::Tmap m;
  std::memset(&m, 0, sizeof(m));
  m.base = base;
  m.tx = TX;
  m.ty = TY;
  const size_t es = ctx->esize;
  const int planes = NV * ctx->nb;
  auto encode = tensor_map_encoder();
  if (encode && ((size_t)ctx->pitch * es) % 16 == 0 && ((size_t)ctx->plane * es) % 16 == 0 &&
      TX + 8 <= 256 && TY + 2 <= 256 && planes <= 256) {
    cuuint64_t dims[3] = {(cuuint64_t)ctx->cfg.nx, (cuuint64_t)ctx->cfg.ny, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)ctx->pitch * es, (cuuint64_t)ctx->plane * es};
    cuuint32_t box[3] = {(cuuint32_t)(TX + 8), (cuuint32_t)(TY + 2), (cuuint32_t)planes};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encode(&m.map, es == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                        3, const_cast<void *>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    m.ok = r == CUDA_SUCCESS;
  }
  ctx->tmaps.push_back(m);
  return ctx->tmaps.back().ok ? &ctx->tmaps.back().map : nullptr;
}

// Run one stage of the integrator.
cudaEvent_t pooled_event(wb_ctx *ctx) {
  if (!ctx->ev_pool.empty()) {
    cudaEvent_t e = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

template <typename R>
int launch_stage_R(wb_ctx *ctx, const StageArgs<R> &A) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ctx->profile) {
    e0 = pooled_event(ctx);
    e1 = pooled_event(ctx);
    CK(cudaEventRecord(e0, ctx->stream));
  }
  // interior tiles of a state buffer are staged by TMA (tensor map for the tile the
  // launch runs)
  int tx = ctx->TX, ty = ctx->TY, cpt = ctx->CPT;
  stage_tile(A, ctx->cfg.order, &tx, &ty, &cpt);
  const CUtensorMap *tm = nullptr;
  for (int b = 0; b < ctx->nbuf; ++b)
    if (A.x == (const R *)ctx->buf[b]) tm = state_tmap(ctx, A.x, tx, ty);
  StageArgs<R> B = A;
  B.use_tma = tm != nullptr;
  CK(launch_stage(B, ctx->cfg.order, ctx->cfg.basis, ctx->TX, ctx->TY, ctx->CPT, tm, ctx->stream));
  if (ctx->profile) {
    CK(cudaEventRecord(e1, ctx->stream));
    ctx->ev.emplace_back(e0, e1);
  }
  return WB_OK;
}

template <typename R>
int ensure_speed(wb_ctx *ctx) {
  if (ctx->speed_valid) return WB_OK;
  CK(cudaMemsetAsync(&ctx->dev->smax[ctx->parity][0], 0, 2 * sizeof(unsigned long long),
                     ctx->stream));
  StageArgs<R> A = base_args<R>(ctx);
  CK(launch_max_speed(A, (const R *)state_buf(ctx, 0), ctx->cfg.order, ctx->cfg.basis,
                      ctx->stream));
  ctx->speed_valid = true;
  return WB_OK;
}

// One time step with the configured integrator.  dt_mode 0: fixed dt; 1: CFL dt.
template <typename R>
int do_step(wb_ctx *ctx, int dt_mode, double dt, double tend) {
  StageArgs<R> A = base_args<R>(ctx);
  A.dt_mode = dt_mode;
  A.dt_fixed = dt;
  A.tend = tend;
  R *U = (R *)state_buf(ctx, 0);
  if (ctx->cfg.integrator == WB_RK2) {
    // 'EQL': w1 = lim(u) + dt L(lim u); u' = 0.5 lim(u) + 0.5 lim(w1) + 0.5 dt L(lim w1)
    R *W1 = (R *)state_buf(ctx, 1), *Un = (R *)state_buf(ctx, 2);
    StageArgs<R> S1 = A;
    S1.x = U;
    S1.o[0].out = W1;
    S1.o[0].beta = R(1);
    S1.o[0].cdt = R(1);
    S1.advance_time = 1;
    int rc = launch_stage_R(ctx, S1);
    if (rc) return rc;
    StageArgs<R> S2 = A;
    S2.x = W1;
    S2.o[0].out = Un;
    S2.o[0].in[0] = U;
    S2.o[0].c[0] = R(0.5);
    S2.o[0].lim[0] = 1;
    S2.o[0].beta = R(0.5);
    S2.o[0].cdt = R(0.5);
    S2.compute_speed = 1;
    rc = launch_stage_R(ctx, S2);
    if (rc) return rc;
    ctx->cur = (ctx->cur + 2) % ctx->nbuf;
  } else {
    // 'RK4' SSP-RK(5,4), 2d/benchmark_2d_dg.f90:683-710, in limit-on-load form
    R *B1 = (R *)state_buf(ctx, 1), *B2 = (R *)state_buf(ctx, 2), *B3 = (R *)state_buf(ctx, 3);
    R *B4 = (R *)state_buf(ctx, 4);
    StageArgs<R> S = A;
    S.x = U;  // stage 1: w1 = u + c1 dt L(u)
    S.o[0].out = B1;
    S.o[0].beta = R(1);
    S.o[0].cdt = R(0.391752226571890);
    S.advance_time = 1;
    int rc = launch_stage_R(ctx, S);
    if (rc) return rc;
    S = A;  // stage 2: w2 = a u + b w1 + c dt L(w1)
    S.x = B1;
    S.o[0].out = B2;
    S.o[0].in[0] = U;
    S.o[0].c[0] = R(0.444370493651235);
    S.o[0].lim[0] = 1;
    S.o[0].beta = R(0.555629506348765);
    S.o[0].cdt = R(0.368410593050371);
    if ((rc = launch_stage_R(ctx, S))) return rc;
    S = A;  // stage 3: w3 = a u + b w2 + c dt L(w2)   (w3 into B1)
    S.x = B2;
    S.o[0].out = B1;
    S.o[0].in[0] = U;
    S.o[0].c[0] = R(0.620101851488403);
    S.o[0].lim[0] = 1;
    S.o[0].beta = R(0.379898148511597);
    S.o[0].cdt = R(0.251891774271694);
    if ((rc = launch_stage_R(ctx, S))) return rc;
    S = A;  // stage 4: w4 = a u + b w3 + c dt L(w3);  w5p = a' u + b' w2 + c' w3 + d' dt L(w3)
    S.x = B1;
    S.o[0].out = B3;
    S.o[0].in[0] = U;
    S.o[0].c[0] = R(0.178079954393132);
    S.o[0].lim[0] = 1;
    S.o[0].beta = R(0.821920045606868);
    S.o[0].cdt = R(0.544974750228521);
    S.o[1].out = B4;
    S.o[1].in[0] = U;
    S.o[1].c[0] = R(0.00683325884039);
    S.o[1].lim[0] = 1;
    S.o[1].in[1] = B2;
    S.o[1].c[1] = R(0.51723167208978);
    S.o[1].lim[1] = 1;
    S.o[1].beta = R(0.12759831133288);
    S.o[1].cdt = R(0.08460416338212);
    if ((rc = launch_stage_R(ctx, S))) return rc;
    S = A;  // stage 5: u' = w5p + 0.34833675773694 w4 + 0.22600748319395 dt L(w4)  (into B2)
    S.x = B3;
    S.o[0].out = B2;
    S.o[0].in[0] = B4;
    S.o[0].c[0] = R(1);
    S.o[0].lim[0] = 0;
    S.o[0].beta = R(0.34833675773694);
    S.o[0].cdt = R(0.22600748319395);
    S.compute_speed = 1;
    if ((rc = launch_stage_R(ctx, S))) return rc;
    ctx->cur = (ctx->cur + 2) % ctx->nbuf;
  }
  ctx->parity ^= 1;
  return WB_OK;
}

int check_dev_err(wb_ctx *ctx) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, &ctx->dev->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (e & 2) return set_err(ctx, WB_ERR_TIMEOUT, "a bounded device wait (tile copy) gave up");
  if (e) return set_err(ctx, WB_ERR_NONPHYSICAL, "non-finite or non-positive density/pressure in a cell mean");
  return WB_OK;
}

// Limited copy of the resident state in kernel precision, in a free state buffer (read
// only for the caller).  Without a limiter the resident state itself is the limited view.
template <typename R>
int limited_copy(wb_ctx *ctx, R **out) {
  if (!(ctx->cfg.limiter && ctx->cfg.order >= 1)) {
    *out = (R *)state_buf(ctx, 0);
    return WB_OK;
  }
  R *dst = (R *)state_buf(ctx, 1);
  CK(cudaMemcpyAsync(dst, state_buf(ctx, 0), ctx->state_bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  if (ctx->cfg.limiter && ctx->cfg.order >= 1) {
    StageArgs<R> A = base_args<R>(ctx);
    CK(launch_limit(A, dst, ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  }
  *out = dst;
  return WB_OK;
}

// Limited FP64 copy (for downloads and norms).
int limited_copy64(wb_ctx *ctx, const double **out) {
  long long n = (long long)NV * ctx->nb * ctx->plane;
  if (is_fp32(ctx)) {
    float *f;
    int rc = limited_copy<float>(ctx, &f);
    if (rc) return rc;
    if ((rc = ensure_scratch(ctx))) return rc;
    CK(launch_f32_to_f64(ctx->scratch64, f, n, ctx->stream));
    *out = ctx->scratch64;
  } else {
    double *d;
    int rc = limited_copy<double>(ctx, &d);
    if (rc) return rc;
    *out = d;
  }
  return WB_OK;
}

// host (double, layout) -> device buffer dst of kernel precision
int host_to_dev(wb_ctx *ctx, const double *h, int layout, void *dst) {
  const size_t rowb = (size_t)ctx->ncell * sizeof(double);
  const int nrow = NV * ctx->nb;
  const int K = ctx->cfg.order;
  if (layout == WB_LAYOUT_SOA) {
    if (!is_fp32(ctx)) return copy_planes(ctx, dst, h, sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    int rc = ensure_scratch(ctx);
    if (rc) return rc;
    if ((rc = copy_planes(ctx, ctx->scratch64, h, sizeof(double), cudaMemcpyHostToDevice, ctx->stream)))
      return rc;
    CK(launch_f64_to_f32((float *)dst, ctx->scratch64, (long long)nrow * ctx->plane, ctx->stream));
    return WB_OK;
  }
  if (ctx->pitch != ctx->cfg.nx) return set_err(ctx, WB_ERR_STATE, "Fortran layout needs unpadded rows");
  int rc = ensure_scratch(ctx);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->scratch64, h, rowb * nrow, cudaMemcpyHostToDevice, ctx->stream));
  if (is_fp32(ctx))
    CK(launch_from_fortran(ctx->scratch64, (float *)dst, ctx->cfg.nx, ctx->cfg.ny, ctx->plane, K, ctx->stream));
  else
    CK(launch_from_fortran(ctx->scratch64, (double *)dst, ctx->cfg.nx, ctx->cfg.ny, ctx->plane, K, ctx->stream));
  return WB_OK;
}

// device buffer src of kernel precision -> host (double, layout)
int dev_to_host(wb_ctx *ctx, const void *src, int layout, double *h) {
  const size_t rowb = (size_t)ctx->ncell * sizeof(double);
  const int nrow = NV * ctx->nb;
  const int K = ctx->cfg.order;
  if (layout == WB_LAYOUT_SOA) {
    const double *s64 = (const double *)src;
    if (is_fp32(ctx)) {
      int rc = ensure_scratch(ctx);
      if (rc) return rc;
      if (src != ctx->scratch64)
        CK(launch_f32_to_f64(ctx->scratch64, (const float *)src, (long long)nrow * ctx->plane, ctx->stream));
      s64 = ctx->scratch64;
    }
    return copy_planes(ctx, h, s64, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  }
  if (ctx->pitch != ctx->cfg.nx) return set_err(ctx, WB_ERR_STATE, "Fortran layout needs unpadded rows");
  int rc = ensure_scratch(ctx);
  if (rc) return rc;
  // gather into the dense Fortran array held in scratch64 (src is a state buffer)
  double *f = ctx->scratch64;
  if (is_fp32(ctx))
    CK(launch_to_fortran((const float *)src, f, ctx->cfg.nx, ctx->cfg.ny, ctx->plane, K, ctx->stream));
  else
    CK(launch_to_fortran((const double *)src, f, ctx->cfg.nx, ctx->cfg.ny, ctx->plane, K, ctx->stream));
  CK(cudaMemcpyAsync(h, f, rowb * nrow, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

// ---- tile cache: lines "precision order basis nx ny tile_x tile_y" (last match wins)
std::string tile_cache_path() {
  const char *e = std::getenv("WB_TILE_CACHE");
  if (e && *e) return e;
  Dl_info info;
  if (dladdr((void *)&wb_create, &info) && info.dli_fname) {
    std::string f = info.dli_fname;
    size_t slash = f.find_last_of('/');
    return (slash == std::string::npos ? std::string(".") : f.substr(0, slash)) + "/tile_cache.txt";
  }
  return "tile_cache.txt";
}
// lines "precision order basis nx ny tile_x tile_y cells_per_thread" (a line without the
// last field means one cell per thread; lines naming shapes not compiled are skipped)
bool tile_cache_lookup(const wb_config &c, int *tx, int *ty, int *cpt) {
  FILE *f = std::fopen(tile_cache_path().c_str(), "r");
  if (!f) return false;
  char line[256];
  bool found = false;
  while (std::fgets(line, sizeof(line), f)) {
    int p, o, b, nx, ny, x, y, k = 1;
    const int n = std::sscanf(line, "%d %d %d %d %d %d %d %d", &p, &o, &b, &nx, &ny, &x, &y, &k);
    if (n >= 7 && p == c.precision && o == c.order && b == c.basis && nx == c.nx &&
        ny == c.ny && tile_supported(p == WB_PREC_FP32, o, b, x, y, k)) {
      *tx = x;
      *ty = y;
      *cpt = k;
      found = true;
    }
  }
  std::fclose(f);
  return found;
}
void tile_cache_store(const wb_config &c, int tx, int ty, int cpt) {
  FILE *f = std::fopen(tile_cache_path().c_str(), "a");
  if (!f) return;
  std::fprintf(f, "%d %d %d %d %d %d %d %d\n", c.precision, c.order, c.basis, c.nx, c.ny, tx, ty,
               cpt);
  std::fclose(f);
}

}  // namespace

extern "C" {

const char *wb_status_string(int s) {
  switch (s) {
  case WB_OK: return "ok";
  case WB_ERR_CONFIG: return "invalid configuration";
  case WB_ERR_CUDA: return "CUDA error";
  case WB_ERR_NONPHYSICAL: return "non-physical state";
  case WB_ERR_TIMEOUT: return "device wait timed out";
  case WB_ERR_ARG: return "bad argument";
  case WB_ERR_NOMEM: return "device allocation failed";
  case WB_ERR_STATE: return "invalid state";
  }
  return "unknown status";
}

int wb_config_default(wb_config *c) {
  if (!c) return WB_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  c->nx = c->ny = 8;  // 2d/parameters_dg_2d.f90:3-4
  c->order = 1;       // mx = my = 2
  c->basis = WB_BASIS_Q;
  c->bc_x = c->bc_y = WB_BC_PERIODIC;  // bc = 1
  c->eq_kind = WB_EQ_ISOTHERMAL;
  c->llf_speed = WB_LLF_MAXABS;
  c->limiter = 1;  // use_limiter = .true.
  c->precision = WB_PREC_FP64;
  c->integrator = WB_RK2;
  c->gamma = 1.4;
  c->gx = 1.0;
  c->gy = 1.0;
  c->rho0 = 1.0;
  c->p0 = 1.0;
  c->kpoly = 1.0;
  c->lx = c->ly = 1.0;  // boxlen_x, boxlen_y
  c->lim_norm = 3.0;    // norm = 3, 2d/limiters.f90:224
  c->lim_M = 0.0;       // M = 0, 2d/parameters_dg_2d.f90:38
  c->lim_tol = 1e-6;    // 2d/limiters.f90:262
  c->cfl = 0.2;         // 2d/parameters_dg_2d.f90:26
  c->pos_eps = 1e-10;   // eps, 2d/parameters_dg_2d.f90:28
  c->riemann = WB_RIEMANN_LLF;  // flux_type = 'llf' (2d/parameters_dg_2d.f90:15)
  return WB_OK;
}

int wb_num_modes(int order, int basis) {
  if (order < 0 || order > KMAX || (basis != 0 && basis != 1)) return WB_ERR_ARG;
  return num_modes(order, basis);
}

int wb_mode_list(int order, int basis, int32_t *dx, int32_t *dy) {
  int n = wb_num_modes(order, basis);
  if (n < 0) return n;
  for (int m = 0; m < n; ++m) {
    if (dx) dx[m] = mode_deg(order, basis, m, 0);
    if (dy) dy[m] = mode_deg(order, basis, m, 1);
  }
  return n;
}

const char *wb_last_error(const wb_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int wb_destroy(wb_ctx *ctx) {
  if (!ctx) return WB_OK;
  cudaSetDevice(ctx->cfg.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (void *&b : ctx->buf) cudaFree(b);
  cudaFree(ctx->scratch64);
  cudaFree(ctx->fxv);
  cudaFree(ctx->fxf);
  cudaFree(ctx->fyv);
  cudaFree(ctx->fyf);
  cudaFree(ctx->fxv64);
  cudaFree(ctx->fxf64);
  cudaFree(ctx->fyv64);
  cudaFree(ctx->fyf64);
  cudaFree(ctx->Td);
  cudaFree(ctx->dev);
  cudaFree(ctx->partial);
  for (auto &p : ctx->ev) {
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->io_init) {
    cudaStreamSynchronize(ctx->s_in);
    cudaStreamSynchronize(ctx->s_out);
    for (int k = 0; k < 2; ++k) {
      cudaFree(ctx->io_in[k]);
      cudaFree(ctx->io_out[k]);
      cudaEventDestroy(ctx->in_ready[k]);
      cudaEventDestroy(ctx->in_free[k]);
      cudaEventDestroy(ctx->out_ready[k]);
      cudaEventDestroy(ctx->out_free[k]);
    }
    cudaStreamDestroy(ctx->s_in);
    cudaStreamDestroy(ctx->s_out);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return WB_OK;
}

}  // extern "C"

namespace wb {
// wb_create with the rows of every plane padded to a multiple of row_align elements (the
// batched form's instances: 16-byte rows for its staging copies); row_align 1 is wb_create.
int ctx_create(const wb_config *cfg, int row_align, wb_ctx **out) {
  if (!cfg || !out || row_align < 1) return WB_ERR_ARG;
  *out = nullptr;
  std::string why;
  int rc = validate(cfg, why);
  wb_ctx *ctx = new wb_ctx();
  ctx->cfg = *cfg;
  if (rc) {
    *out = ctx;  // returned so the caller can read wb_last_error; must still be destroyed
    return set_err(ctx, rc, why);
  }
  *out = ctx;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return set_err(ctx, WB_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (cfg->device < 0 || cfg->device >= ndev) return set_err(ctx, WB_ERR_CONFIG, "bad device ordinal");
  CK(cudaSetDevice(cfg->device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  const int K = cfg->order;
  ctx->nq = K + 1;
  ctx->nb = num_modes(K, cfg->basis);
  ctx->ncell = (long long)cfg->nx * cfg->ny;
  ctx->pitch = (cfg->nx + row_align - 1) / row_align * row_align;
  ctx->plane = ((long long)ctx->pitch * cfg->ny + 63) / 64 * 64;
  ctx->esize = is_fp32(ctx) ? sizeof(float) : sizeof(double);
  ctx->state_bytes = (size_t)NV * ctx->nb * ctx->plane * ctx->esize;
  ctx->nbuf = cfg->integrator == WB_RK2 ? 3 : 5;
  if (cfg->tile_x > 0) {
    ctx->TX = cfg->tile_x;
    ctx->TY = cfg->tile_y;
    ctx->CPT = cfg->cells_per_thread > 0 ? cfg->cells_per_thread : 1;
  } else if (is_fp32(ctx)) {
    // untuned default: the measured best on large grids -- 32x8 at one cell per thread for
    // degree 2, 32x16 at two cells per thread for degrees 0 and 1 (where compiled)
    ctx->TX = 32;
    ctx->TY = 8;
    if (K <= 1 && tile_supported(1, K, cfg->basis, 32, 16, 2)) {
      ctx->TY = 16;
      ctx->CPT = 2;
    }
  } else {
    ctx->TX = 16;
    ctx->TY = 8;
  }
  if (cfg->tile_x <= 0) tile_cache_lookup(*cfg, &ctx->TX, &ctx->TY, &ctx->CPT);
  // basis tables (constant memory of both precisions' kernels, FP64 copy in global)
  Tab1D<double> t64[KMAX + 1];
  Tab1D<float> t32[KMAX + 1];
  make_tab1d(t64);
  convert_tabs<float>(t64, t32, KMAX + 1);
  CK(upload_tables(t32, t64));
  if ((rc = dalloc(ctx, &ctx->Td, sizeof(t64)))) return rc;
  CK(cudaMemcpy(ctx->Td, t64, sizeof(t64), cudaMemcpyHostToDevice));
  // equilibrium factor tables
  if ((rc = build_eq_tables(ctx, t64[K].xq))) return rc;
  for (int b = 0; b < ctx->nbuf; ++b) {
    if ((rc = dalloc(ctx, (char **)&ctx->buf[b], ctx->state_bytes))) return rc;
    CK(cudaMemsetAsync(ctx->buf[b], 0, ctx->state_bytes, ctx->stream));
  }
  if ((rc = dalloc(ctx, &ctx->dev, sizeof(DevState)))) return rc;
  CK(cudaMemsetAsync(ctx->dev, 0, sizeof(DevState), ctx->stream));
  if ((rc = dalloc(ctx, (char **)&ctx->partial, diag_partial_bytes(cfg->nx, cfg->ny)))) return rc;
  ctx->diag_out = ctx->partial;  // final results go to the front, partials after 64 doubles
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}
}  // namespace wb

extern "C" {

int wb_create(const wb_config *cfg, wb_ctx **out) { return ctx_create(cfg, 1, out); }

int wb_upload_state(wb_ctx *ctx, const double *delta, int32_t layout) {
  if (!ctx || !delta) return WB_ERR_ARG;
  if (layout != WB_LAYOUT_SOA && layout != WB_LAYOUT_FORTRAN) return set_err(ctx, WB_ERR_ARG, "bad layout");
  if (layout == WB_LAYOUT_FORTRAN && ctx->cfg.basis != WB_BASIS_Q)
    return set_err(ctx, WB_ERR_ARG, "the Fortran layout needs the tensor basis");
  CK(cudaSetDevice(ctx->cfg.device));
  int rc = host_to_dev(ctx, delta, layout, state_buf(ctx, 0));
  if (rc) return rc;
  ctx->speed_valid = false;
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

int wb_download_state(wb_ctx *ctx, double *delta, int32_t layout) {
  if (!ctx || !delta) return WB_ERR_ARG;
  if (layout != WB_LAYOUT_SOA && layout != WB_LAYOUT_FORTRAN) return set_err(ctx, WB_ERR_ARG, "bad layout");
  if (layout == WB_LAYOUT_FORTRAN && ctx->cfg.basis != WB_BASIS_Q)
    return set_err(ctx, WB_ERR_ARG, "the Fortran layout needs the tensor basis");
  CK(cudaSetDevice(ctx->cfg.device));
  int rc;
  if (is_fp32(ctx)) {
    float *f;
    if ((rc = limited_copy<float>(ctx, &f))) return rc;
    if ((rc = dev_to_host(ctx, f, layout, delta))) return rc;
  } else {
    double *d;
    if ((rc = limited_copy<double>(ctx, &d))) return rc;
    if ((rc = dev_to_host(ctx, d, layout, delta))) return rc;
  }
  return check_dev_err(ctx);
}

int wb_download_state_raw(wb_ctx *ctx, void *delta) {
  if (!ctx || !delta) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  const size_t es = is_fp32(ctx) ? sizeof(float) : sizeof(double);
  int rc = copy_planes(ctx, delta, state_buf(ctx, 0), es, cudaMemcpyDeviceToHost, ctx->stream);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return check_dev_err(ctx);
}

int wb_upload_state_f32(wb_ctx *ctx, const float *delta) {
  if (!ctx || !delta) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  const int nrow = NV * ctx->nb;
  int rc;
  if (is_fp32(ctx)) {
    if ((rc = copy_planes(ctx, state_buf(ctx, 0), delta, sizeof(float), cudaMemcpyHostToDevice,
                          ctx->stream)))
      return rc;
  } else {
    float *tmp = (float *)state_buf(ctx, 1);  // free buffer, large enough for FP32
    if ((rc = copy_planes(ctx, tmp, delta, sizeof(float), cudaMemcpyHostToDevice, ctx->stream)))
      return rc;
    CK(launch_f32_to_f64((double *)state_buf(ctx, 0), tmp, (long long)nrow * ctx->plane, ctx->stream));
  }
  ctx->speed_valid = false;
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

int wb_download_state_f32(wb_ctx *ctx, float *delta) {
  if (!ctx || !delta) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  const int nrow = NV * ctx->nb;
  int rc;
  if (is_fp32(ctx)) {
    float *f;
    if ((rc = limited_copy<float>(ctx, &f))) return rc;
    if ((rc = copy_planes(ctx, delta, f, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream)))
      return rc;
  } else {
    double *d;
    if ((rc = limited_copy<double>(ctx, &d))) return rc;
    float *tmp = (float *)state_buf(ctx, 2);
    CK(launch_f64_to_f32(tmp, d, (long long)nrow * ctx->plane, ctx->stream));
    if ((rc = copy_planes(ctx, delta, tmp, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream)))
      return rc;
  }
  return check_dev_err(ctx);
}

int wb_init_perturbation(wb_ctx *ctx, const wb_perturbation *ic) {
  if (!ctx || !ic) return WB_ERR_ARG;
  if (ic->kind < 0 || ic->kind > 2 || ic->nmodes < 0 || ic->nmodes > 32)
    return set_err(ctx, WB_ERR_ARG, "bad perturbation");
  if (ic->kind == 1 && !(ic->sigma > 0.0)) return set_err(ctx, WB_ERR_ARG, "sigma must be > 0");
  CK(cudaSetDevice(ctx->cfg.device));
  IcArgs I;
  std::memset(&I, 0, sizeof(I));
  I.kind = ic->kind;
  I.nmodes = ic->nmodes;
  I.amp = ic->amp;
  I.xc = ic->xc;
  I.yc = ic->yc;
  I.sigma = ic->sigma;
  for (int m = 0; m < 32; ++m) {
    I.kx[m] = ic->kx[m];
    I.ky[m] = ic->ky[m];
    I.pu[m] = ic->phase_u[m];
    I.pv[m] = ic->phase_v[m];
    I.wt[m] = ic->weight[m];
  }
  AuxArgs A = aux_args(ctx);
  if (is_fp32(ctx))
    CK(launch_init_ic(A, I, ctx->Td, (float *)state_buf(ctx, 0), ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  else
    CK(launch_init_ic(A, I, ctx->Td, (double *)state_buf(ctx, 0), ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  CK(cudaMemsetAsync(ctx->dev, 0, sizeof(DevState), ctx->stream));
  ctx->parity = 0;
  ctx->speed_valid = false;
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

int wb_device_state(wb_ctx *ctx, void **dptr, size_t *plane_stride) {
  if (!ctx || !dptr) return WB_ERR_ARG;
  *dptr = state_buf(ctx, 0);
  if (plane_stride) *plane_stride = (size_t)ctx->plane;
  return WB_OK;
}

int wb_compute_update(wb_ctx *ctx, const double *delta_u, double *dudt, int32_t layout) {
  if (!ctx || !delta_u || !dudt) return WB_ERR_ARG;
  if (layout != WB_LAYOUT_SOA && layout != WB_LAYOUT_FORTRAN) return set_err(ctx, WB_ERR_ARG, "bad layout");
  if (layout == WB_LAYOUT_FORTRAN && ctx->cfg.basis != WB_BASIS_Q)
    return set_err(ctx, WB_ERR_ARG, "the Fortran layout needs the tensor basis");
  CK(cudaSetDevice(ctx->cfg.device));
  void *X = state_buf(ctx, 1), *Y = state_buf(ctx, 2);
  int rc = host_to_dev(ctx, delta_u, layout, X);
  if (rc) return rc;
  if (is_fp32(ctx)) {
    StageArgs<float> A = base_args<float>(ctx);
    A.x = (const float *)X;
    A.lim_y = 0;
    A.dt_fixed = 1.0;
    A.o[0].out = (float *)Y;
    A.o[0].beta = 0.0f;
    A.o[0].cdt = 1.0f;
    if ((rc = launch_stage_R(ctx, A))) return rc;
  } else {
    StageArgs<double> A = base_args<double>(ctx);
    A.x = (const double *)X;
    A.lim_y = 0;
    A.dt_fixed = 1.0;
    A.o[0].out = (double *)Y;
    A.o[0].beta = 0.0;
    A.o[0].cdt = 1.0;
    if ((rc = launch_stage_R(ctx, A))) return rc;
  }
  if ((rc = dev_to_host(ctx, Y, layout, dudt))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

int wb_apply_limiter(wb_ctx *ctx) {
  if (!ctx) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  if (ctx->cfg.limiter && ctx->cfg.order >= 1) {
    if (is_fp32(ctx))
      CK(launch_limit(base_args<float>(ctx), (float *)state_buf(ctx, 0), ctx->cfg.order, ctx->cfg.basis, ctx->stream));
    else
      CK(launch_limit(base_args<double>(ctx), (double *)state_buf(ctx, 0), ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

int wb_max_speed(wb_ctx *ctx, double *sx, double *sy) {
  if (!ctx) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  ctx->speed_valid = false;
  int rc = is_fp32(ctx) ? ensure_speed<float>(ctx) : ensure_speed<double>(ctx);
  if (rc) return rc;
  unsigned long long bits[2];
  CK(cudaMemcpyAsync(bits, &ctx->dev->smax[ctx->parity][0], sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double v[2];
  std::memcpy(v, bits, sizeof(v));
  if (sx) *sx = v[0];
  if (sy) *sy = v[1];
  return check_dev_err(ctx);
}

static int step_impl(wb_ctx *ctx, int nsteps, int dt_mode, double dt, double tend) {
  int rc;
  if (is_fp32(ctx)) {
    if (dt_mode == 1 && (rc = ensure_speed<float>(ctx))) return rc;
    for (int n = 0; n < nsteps; ++n)
      if ((rc = do_step<float>(ctx, dt_mode, dt, tend))) return rc;
  } else {
    if (dt_mode == 1 && (rc = ensure_speed<double>(ctx))) return rc;
    for (int n = 0; n < nsteps; ++n)
      if ((rc = do_step<double>(ctx, dt_mode, dt, tend))) return rc;
  }
  return WB_OK;
}

int wb_step(wb_ctx *ctx, int32_t nsteps, double dt) {
  if (!ctx || nsteps < 0) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  return step_impl(ctx, nsteps, dt > 0.0 ? 0 : 1, dt, -1.0);
}

int wb_autotune(wb_ctx *ctx, int32_t steps, int32_t *tile_x, int32_t *tile_y,
                int32_t *cells_per_thread) {
  if (!ctx || steps < 1) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  // every compiled (tile, cells per thread) of this precision, degree and basis
  int cand[16][3];
  const int ncand = tile_candidates(is_fp32(ctx), ctx->cfg.order, ctx->cfg.basis, cand, 16);
  // save the run so every candidate starts from the same state
  void *backup = nullptr;
  int rc = dalloc(ctx, (char **)&backup, ctx->state_bytes);
  if (rc) return rc;
  DevState saved;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(backup, state_buf(ctx, 0), ctx->state_bytes, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy(&saved, ctx->dev, sizeof(saved), cudaMemcpyDeviceToHost));
  const int cur0 = ctx->cur, par0 = ctx->parity;
  const bool sv0 = ctx->speed_valid;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 0.0f;
  int bx = ctx->TX, by = ctx->TY, bc = ctx->CPT;
  for (int k = 0; k < ncand && rc == WB_OK; ++k) {
    ctx->cur = cur0;
    ctx->parity = par0;
    ctx->speed_valid = sv0;
    CK(cudaMemcpy(state_buf(ctx, 0), backup, ctx->state_bytes, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(ctx->dev, &saved, sizeof(saved), cudaMemcpyHostToDevice));
    ctx->TX = cand[k][0];
    ctx->TY = cand[k][1];
    ctx->CPT = cand[k][2];
    if ((rc = step_impl(ctx, 1, 1, 0.0, -1.0))) break;  // warm-up (first launch set-up)
    CK(cudaEventRecord(e0, ctx->stream));
    if ((rc = step_impl(ctx, steps, 1, 0.0, -1.0))) break;
    CK(cudaEventRecord(e1, ctx->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (k == 0 || ms < best) {
      best = ms;
      bx = ctx->TX;
      by = ctx->TY;
      bc = ctx->CPT;
    }
  }
  ctx->cur = cur0;
  ctx->parity = par0;
  ctx->speed_valid = sv0;
  cudaMemcpy(state_buf(ctx, 0), backup, ctx->state_bytes, cudaMemcpyDeviceToDevice);
  cudaMemcpy(ctx->dev, &saved, sizeof(saved), cudaMemcpyHostToDevice);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(backup);
  if (rc) return rc;
  ctx->TX = bx;
  ctx->TY = by;
  ctx->CPT = bc;
  tile_cache_store(ctx->cfg, bx, by, bc);
  if (tile_x) *tile_x = bx;
  if (tile_y) *tile_y = by;
  if (cells_per_thread) *cells_per_thread = bc;
  return WB_OK;
}

int wb_sync(wb_ctx *ctx) {
  if (!ctx) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  if (ctx->io_init) {
    CK(cudaStreamSynchronize(ctx->s_in));
    CK(cudaStreamSynchronize(ctx->s_out));
  }
  return check_dev_err(ctx);
}

int wb_set_equilibrium(wb_ctx *ctx, int32_t kind, double gx, double gy, const double *params) {
  if (!ctx) return WB_ERR_ARG;
  wb_config c = ctx->cfg;
  c.eq_kind = kind;
  c.gx = gx;
  c.gy = gy;
  if (params) {
    c.rho0 = params[0];
    c.p0 = params[1];
    c.kpoly = params[2];
  }
  std::string why;
  if (int v = validate(&c, why)) return set_err(ctx, v, why);
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaStreamSynchronize(ctx->stream));  // in-flight stages read the old tables
  if (ctx->io_init) {
    CK(cudaStreamSynchronize(ctx->s_in));
    CK(cudaStreamSynchronize(ctx->s_out));
  }
  ctx->cfg = c;
  Tab1D<double> t64[KMAX + 1];
  make_tab1d(t64);
  int rc = build_eq_tables(ctx, t64[ctx->cfg.order].xq);
  if (rc) return rc;
  ctx->speed_valid = false;
  return WB_OK;
}

int wb_selftest_wait_timeout(wb_ctx *ctx, int32_t polls) {
  if (!ctx || polls < 1) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  int e = 0;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(launch_wait_selftest(&ctx->dev->err, polls, ctx->stream));
  CK(cudaMemcpyAsync(&e, &ctx->dev->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemsetAsync(&ctx->dev->err, 0, sizeof(int), ctx->stream));  // context stays usable
  CK(cudaStreamSynchronize(ctx->stream));
  return (e & 2) ? WB_ERR_TIMEOUT : WB_OK;
}

int wb_step_io_f32(wb_ctx *ctx, const float *in, float *out, int32_t nsteps, double dt) {
  if (!ctx || !in || !out || nsteps < 0) return WB_ERR_ARG;
  if (!is_fp32(ctx)) return set_err(ctx, WB_ERR_STATE, "wb_step_io_f32 needs an FP32 context");
  CK(cudaSetDevice(ctx->cfg.device));
  if (!ctx->io_init) {
    CK(cudaStreamCreateWithFlags(&ctx->s_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->s_out, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      int rc;
      if ((rc = dalloc(ctx, (char **)&ctx->io_in[k], ctx->state_bytes))) return rc;
      if ((rc = dalloc(ctx, (char **)&ctx->io_out[k], ctx->state_bytes))) return rc;
      CK(cudaEventCreateWithFlags(&ctx->in_ready[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->in_free[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->out_ready[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->out_free[k], cudaEventDisableTiming));
    }
    ctx->io_init = true;
  }
  const int k = ctx->io_k & 1;
  ++ctx->io_k;
  // 1. input: host -> staging buffer k (free once the compute stream took its last input)
  CK(cudaStreamWaitEvent(ctx->s_in, ctx->in_free[k], 0));
  int rc = copy_planes(ctx, ctx->io_in[k], in, sizeof(float), cudaMemcpyHostToDevice, ctx->s_in);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->in_ready[k], ctx->s_in));
  // 2. compute stream: take the input as the state, step, leave the limited result
  CK(cudaStreamWaitEvent(ctx->stream, ctx->in_ready[k], 0));
  // device-side copies run on the SMs: the copy engines are busy with the host transfers
  CK(launch_copy_device(state_buf(ctx, 0), ctx->io_in[k], ctx->state_bytes, ctx->stream));
  CK(cudaEventRecord(ctx->in_free[k], ctx->stream));
  ctx->speed_valid = false;
  rc = step_impl(ctx, nsteps, dt > 0.0 ? 0 : 1, dt, -1.0);
  if (rc) return rc;
  CK(cudaStreamWaitEvent(ctx->stream, ctx->out_free[k], 0));
  CK(launch_copy_device(ctx->io_out[k], state_buf(ctx, 0), ctx->state_bytes, ctx->stream));
  if (ctx->cfg.limiter && ctx->cfg.order >= 1) {
    StageArgs<float> A = base_args<float>(ctx);
    CK(launch_limit(A, (float *)ctx->io_out[k], ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  }
  CK(cudaEventRecord(ctx->out_ready[k], ctx->stream));
  // 3. output: staging buffer k -> host
  CK(cudaStreamWaitEvent(ctx->s_out, ctx->out_ready[k], 0));
  if ((rc = copy_planes(ctx, out, ctx->io_out[k], sizeof(float), cudaMemcpyDeviceToHost, ctx->s_out)))
    return rc;
  CK(cudaEventRecord(ctx->out_free[k], ctx->s_out));
  return WB_OK;
}

int wb_get_time(wb_ctx *ctx, double *t, int64_t *steps) {
  if (!ctx) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  DevState h;
  CK(cudaMemcpyAsync(&h, ctx->dev, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (t) *t = h.t[ctx->parity];
  if (steps) *steps = h.nstep[ctx->parity];
  return WB_OK;
}

int wb_write_dat(wb_ctx *ctx, const char *path, int32_t var) {
  if (!ctx || !path || var < 1 || var > 4) return WB_ERR_ARG;
  const wb_config &g = ctx->cfg;
  std::vector<double> d((size_t)NV * ctx->nb * ctx->ncell);
  int rc = wb_download_state(ctx, d.data(), WB_LAYOUT_SOA);
  if (rc) return rc;
  Tab1D<double> t64[KMAX + 1];
  make_tab1d(t64);
  const Tab1D<double> &T = t64[g.order];
  EqParams ep{g.eq_kind, g.gamma, g.gx, g.gy, g.rho0, g.p0, g.kpoly};
  const double dx = g.lx / g.nx, dy = g.ly / g.ny, gm1 = g.gamma - 1.0;
  FILE *f = std::fopen(path, "w");
  if (!f) return set_err(ctx, WB_ERR_ARG, std::string("cannot open ") + path);
  char num[16];
  for (int i = 0; i < g.nx; ++i)
    for (int j = 0; j < g.ny; ++j) {
      const size_t cell = (size_t)j * g.nx + i;
      const double x = ((double)i + 0.5) * dx + dx / 2.0 * T.xq[0];
      const double y = ((double)j + 0.5) * dy + dy / 2.0 * T.xq[0];
      double re, pe;
      eq_combine(ep, eq_factor_x(ep, x), eq_factor_y(ep, y), &re, &pe);
      double u[NV];
      for (int v = 0; v < NV; ++v) {
        double s = 0.0;
        for (int m = 0; m < ctx->nb; ++m)
          s += d[((size_t)v * ctx->nb + m) * ctx->ncell + cell] *
               T.B[mode_deg(g.order, g.basis, m, 0)][0] * T.B[mode_deg(g.order, g.basis, m, 1)][0];
        u[v] = s;
      }
      // w - w_eq of compute_primitive (2d/benchmark_2d_dg.f90:891-903) at rest: the
      // pressure difference taken without the cancellation p(u_eq + d) - p_eq
      const double rho = re + u[0], vx = u[1] / rho, vy = u[2] / rho;
      const double w[NV] = {u[0], vx, vy, gm1 * (u[3] - 0.5 * rho * (vx * vx + vy * vy))};
      // fields separated by the 1X of the format; Fortran ends the record at the last
      // field, with no trailing blank
      fortran_1pe12_5(x, num);
      std::fprintf(f, "%s", num);
      fortran_1pe12_5(y, num);
      std::fprintf(f, " %s", num);
      for (int v = var - 1; v < NV; ++v) {
        fortran_1pe12_5(w[v], num);
        std::fprintf(f, " %s", num);
      }
      std::fprintf(f, "\n");
    }
  std::fclose(f);
  return WB_OK;
}

int wb_set_time(wb_ctx *ctx, double t, int64_t steps) {
  if (!ctx || !(t >= 0.0) || steps < 0) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  DevState h;
  CK(cudaMemcpyAsync(&h, ctx->dev, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  h.t[ctx->parity] = t;
  h.nstep[ctx->parity] = steps;
  CK(cudaMemcpyAsync(ctx->dev, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

int wb_evolve(wb_ctx *ctx, double tend, int32_t max_steps, int32_t *steps_done, double *t_out) {
  if (!ctx || max_steps < 0) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  double t;
  int64_t n0, n;
  int rc = wb_get_time(ctx, &t, &n0);
  if (rc) return rc;
  int launched = 0;
  int chunk = 4;
  while (t < tend && launched < max_steps) {
    int now = std::min(chunk, max_steps - launched);
    if ((rc = step_impl(ctx, now, 1, 0.0, tend))) return rc;
    launched += now;
    if ((rc = wb_get_time(ctx, &t, &n))) return rc;
    if ((rc = check_dev_err(ctx))) return rc;
    if (chunk < 256) chunk *= 2;
  }
  if ((rc = wb_get_time(ctx, &t, &n))) return rc;
  if (steps_done) *steps_done = (int32_t)(n - n0);
  if (t_out) *t_out = t;
  return check_dev_err(ctx);
}

int wb_norms(wb_ctx *ctx, wb_ctx *other, double l1[4], double linf[4], double l2[4]) {
  if (!ctx) return WB_ERR_ARG;
  if (other && (other->cfg.nx != ctx->cfg.nx || other->cfg.ny != ctx->cfg.ny ||
                other->cfg.order != ctx->cfg.order || other->cfg.basis != ctx->cfg.basis ||
                other->cfg.device != ctx->cfg.device || other->pitch != ctx->pitch))
    return set_err(ctx, WB_ERR_ARG, "norms need contexts with the same grid, basis and device");
  CK(cudaSetDevice(ctx->cfg.device));
  const double *b = nullptr;
  int rc;
  if (other) {
    if ((rc = limited_copy64(other, &b))) return set_err(ctx, rc, other->err);
    CK(cudaStreamSynchronize(other->stream));
  }
  const double *a;
  if ((rc = limited_copy64(ctx, &a))) return rc;
  // limited_copy64 of an FP32 context uses scratch64; when both are FP32 the two copies
  // live in different contexts, so they never alias.
  CK(launch_norms(aux_args(ctx), ctx->Td, a, b, ctx->partial + 64, ctx->diag_out,
                  ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  double h[12];
  CK(cudaMemcpyAsync(h, ctx->diag_out, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int v = 0; v < 4; ++v) {
    if (l1) l1[v] = h[v];
    if (l2) l2[v] = std::sqrt(h[4 + v]);
    if (linf) linf[v] = h[8 + v];
  }
  return WB_OK;
}

int wb_get_stream(wb_ctx *ctx, void **stream) {
  if (!ctx || !stream) return WB_ERR_ARG;
  *stream = (void *)ctx->stream;
  return WB_OK;
}

int wb_profile_stages(wb_ctx *ctx, int32_t on) {
  if (!ctx) return WB_ERR_ARG;
  ctx->profile = on != 0;
  return WB_OK;
}

int wb_stage_stats(wb_ctx *ctx, double *total_ms, int64_t *launches) {
  if (!ctx) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  CK(cudaStreamSynchronize(ctx->stream));
  double tot = 0.0;
  for (auto &p : ctx->ev) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, p.first, p.second));
    tot += ms;
    ctx->ev_pool.push_back(p.first);
    ctx->ev_pool.push_back(p.second);
  }
  if (total_ms) *total_ms = tot;
  if (launches) *launches = (int64_t)ctx->ev.size();
  ctx->ev.clear();
  return WB_OK;
}

int wb_conserved_sums(wb_ctx *ctx, double sums[4]) {
  if (!ctx || !sums) return WB_ERR_ARG;
  CK(cudaSetDevice(ctx->cfg.device));
  AuxArgs A = aux_args(ctx);
  if (is_fp32(ctx))
    CK(launch_sums(A, ctx->Td, (const float *)state_buf(ctx, 0), ctx->partial + 64, ctx->diag_out,
                   ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  else
    CK(launch_sums(A, ctx->Td, (const double *)state_buf(ctx, 0), ctx->partial + 64, ctx->diag_out,
                   ctx->cfg.order, ctx->cfg.basis, ctx->stream));
  CK(cudaMemcpyAsync(sums, ctx->diag_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return WB_OK;
}

}  // extern "C"

// ------------------------------------------------ context internals for the batch
namespace wb {

int ctx_rk2_stage_args(wb_ctx *ctx, int phase, int dt_mode, double dt, StageArgs<float> out[2]) {
  if (!is_fp32(ctx) || ctx->cfg.integrator != WB_RK2) return WB_ERR_CONFIG;
  const int cur0 = ctx->cur, par0 = ctx->parity;
  ctx->cur = (cur0 + 2 * phase) % ctx->nbuf;
  ctx->parity = (par0 + phase) & 1;
  StageArgs<float> A = base_args<float>(ctx);
  A.dt_mode = dt_mode;
  A.dt_fixed = dt;
  float *U = (float *)state_buf(ctx, 0), *W1 = (float *)state_buf(ctx, 1);
  float *Un = (float *)state_buf(ctx, 2);
  out[0] = A;
  out[0].x = U;
  out[0].o[0].out = W1;
  out[0].o[0].beta = 1.0f;
  out[0].o[0].cdt = 1.0f;
  out[0].advance_time = 1;
  out[1] = A;
  out[1].x = W1;
  out[1].o[0].out = Un;
  out[1].o[0].in[0] = U;
  out[1].o[0].c[0] = 0.5f;
  out[1].o[0].lim[0] = 1;
  out[1].o[0].beta = 0.5f;
  out[1].o[0].cdt = 0.5f;
  out[1].compute_speed = 1;
  ctx->cur = cur0;
  ctx->parity = par0;
  return WB_OK;
}
const float *ctx_state_f32(wb_ctx *c) { return (const float *)state_buf(c, 0); }
const CUtensorMap *ctx_state_tmap(wb_ctx *c, const void *base, int TX, int TY) {
  return state_tmap(c, base, TX, TY);
}
DevState *ctx_dev_state(wb_ctx *c) { return c->dev; }
void ctx_tile(wb_ctx *c, int *tx, int *ty, int *cpt) {
  *tx = c->TX;
  *ty = c->TY;
  *cpt = c->CPT;
}
void ctx_advance(wb_ctx *c, int n) {
  c->cur = (c->cur + 2 * n) % c->nbuf;
  c->parity = (c->parity + n) & 1;
}
void ctx_set_speed_valid(wb_ctx *c, bool v) { c->speed_valid = v; }
bool ctx_speed_valid(wb_ctx *c) { return c->speed_valid; }
int ctx_parity(wb_ctx *c) { return c->parity; }
size_t ctx_dofs(wb_ctx *c) { return (size_t)NV * c->nb * c->ncell; }

}  // namespace wb
