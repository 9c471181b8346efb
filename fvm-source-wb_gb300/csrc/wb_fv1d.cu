// wb_fv1d.cu -- 1D well-balanced finite-volume step (the fvm.f90 / benchmark_1d.f90 path)
// on the device, FP64.  Two schemes: 'EQL' (below) and the hydrostatic reconstruction
// 'WB1' (rhs_wb1).
//
// Scheme (compute_update 'EQL', benchmark_1d.f90:263-377): face states are the
// equilibrium at the face plus the perturbation of the adjacent cell, reconstructed
// with minmod slopes (minmod of limiters.f90:1-21); LLF flux (:438-451) minus the
// equilibrium flux at the face; source -rho g, -m g minus its equilibrium part.  The
// time loop of evolve (:200-261) with a true SSP-RK2 second stage and dt = cfl dx /
// max(|u|+c) clipped at tend runs inside one CTA (the grid is small: N = 256 in the
// published configuration), so a whole run is one launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wb_capi.h"
#include "wb_tables.h"

namespace {

struct Fv1dArgs {
  int nx, bc, limiter, max_steps, rhs_only, scheme;
  double dx, gamma, g, cfl, tend;
  double *d, *w1, *fh, *L;       // state, stage state, face fluxes [(nx+1)*3], rhs [nx*3]
  const double *re, *pe;         // equilibrium at centres
  const double *ref, *pef;       // equilibrium at faces
  double *t;                     // in/out simulated time
  int *steps;                    // out steps taken
};

__device__ __forceinline__ int map1(int i, int n, int bc) {
  if (i >= 0 && i < n) return i;
  if (bc == WB_BC_PERIODIC) return ((i % n) + n) % n;
  return i < 0 ? 0 : n - 1;
}
__device__ __forceinline__ double mm3(double x, double y, double z) {
  double s = copysign(1.0, x);
  if (copysign(1.0, y) == s && copysign(1.0, z) == s) return s * fmin(fmin(fabs(x), fabs(y)), fabs(z));
  return 0.0;
}
__device__ __forceinline__ void prim1(double g, const double *u, double *w) {
  w[0] = u[0];
  w[1] = u[1] / w[0];
  w[2] = (g - 1.0) * (u[2] - 0.5 * w[0] * w[1] * w[1]);
}
__device__ __forceinline__ void flux1(double g, const double *u, double *f) {
  double w[3];
  prim1(g, u, w);
  f[0] = w[1] * u[0];
  f[1] = w[1] * u[1] + w[2];
  f[2] = w[1] * u[2] + w[2] * w[1];
}
__device__ __forceinline__ double speed1(double g, const double *u) {
  double w[3];
  prim1(g, u, w);
  return fabs(w[1]) + sqrt(g * fmax(w[2], 1e-10) / fmax(w[0], 1e-10));
}
__device__ __forceinline__ double slope(const Fv1dArgs &A, const double *d, int i, int v) {
  if (!A.limiter) return 0.0;
  if (A.bc != WB_BC_PERIODIC && (i < 0 || i >= A.nx)) return 0.0;
  double c = d[3 * map1(i, A.nx, A.bc) + v];
  double dp = d[3 * map1(i + 1, A.nx, A.bc) + v] - c;
  double dm = c - d[3 * map1(i - 1, A.nx, A.bc) + v];
  return mm3(dp, dm, dm);
}

// 'WB1' face states of cell i (compute_update_sr, benchmark_1d.f90:553-747): the cell's
// specific enthalpy h = p/rho (1 + 1/(gamma-1)) and K = p/rho^gamma (default-real floor
// 1e-5, :611,619) carried to its faces along h + Phi = const (Phi = g x, :615-616), with
// the cell velocity (:631-635).  w receives the cell's primitive state.
__device__ void wb1_face_states(const Fv1dArgs &A, const double *d, int i, double *uL,
                                double *uR, double &pL, double &pR, double *w) {
  const double g = A.gamma, fl = (double)1e-5f;
  const double u[3] = {A.re[i] + d[3 * i], d[3 * i + 1], A.pe[i] / (g - 1.0) + d[3 * i + 2]};
  prim1(g, u, w);
  const double h = fmax(w[2], fl) / fmax(fl, w[0]) * (1 + 1. / (g - 1));
  const double xc = ((double)i + 0.5) * A.dx, xl = (double)i * A.dx, xr = (double)(i + 1) * A.dx;
  const double h0l = h + A.g * xc - A.g * xl, h0r = h + A.g * xc - A.g * xr;
  const double K = fmax(fl, w[2]) / pow(fmax(fl, w[0]), g);
  const double rl = pow((1. / K) * (g - 1) / g * h0l, 1 / (g - 1));
  const double rr = pow((1. / K) * (g - 1) / g * h0r, 1 / (g - 1));
  pL = pow(1. / K, 1 / (g - 1)) * pow((g - 1) / g * h0l, g / (g - 1));
  pR = pow(1. / K, 1 / (g - 1)) * pow((g - 1) / g * h0r, g / (g - 1));
  uL[0] = rl;
  uL[1] = rl * w[1];
  uL[2] = pL / (g - 1.0) + 0.5 * rl * w[1] * w[1];
  uR[0] = rr;
  uR[1] = rr * w[1];
  uR[2] = pR / (g - 1.0) + 0.5 * rr * w[1] * w[1];
}

// 'WB1' L(d): LLF of the adjacent face states on the interior faces (:642-666), source
// (0, (p_right - p_left)/dx, -rho v g (x+ - x-)/(2 dx)) (get_source_rg :409-434), the end
// cells take their neighbour's update (:741-742).
__device__ void rhs_wb1(const Fv1dArgs &A, const double *d) {
  const int nx = A.nx;
  for (int f = 1 + threadIdx.x; f < nx; f += blockDim.x) {
    double aL[3], aR[3], bL[3], bR[3], p1, p2, p3, p4, w[3], fa[3], fb[3];
    wb1_face_states(A, d, f - 1, aL, aR, p1, p2, w);
    wb1_face_states(A, d, f, bL, bR, p3, p4, w);
    flux1(A.gamma, aR, fa);
    flux1(A.gamma, bL, fb);
    const double cmax = fmax(speed1(A.gamma, aR), speed1(A.gamma, bL));
    for (int v = 0; v < 3; ++v) A.fh[3 * f + v] = 0.5 * (fb[v] + fa[v]) - 0.5 * cmax * (bL[v] - aR[v]);
  }
  __syncthreads();
  for (int i = 1 + threadIdx.x; i < nx - 1; i += blockDim.x) {
    double uL[3], uR[3], pL, pR, w[3];
    wb1_face_states(A, d, i, uL, uR, pL, pR, w);
    const double xm = ((double)(i - 1) + 0.5) * A.dx, xp = ((double)(i + 1) + 0.5) * A.dx;
    const double s[3] = {0.0, (pR - pL) / A.dx, -w[0] * w[1] * A.g * (xp - xm) / (2 * A.dx)};
    for (int v = 0; v < 3; ++v) A.L[3 * i + v] = -(A.fh[3 * (i + 1) + v] - A.fh[3 * i + v]) / A.dx + s[v];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int v = threadIdx.x;
    A.L[v] = A.L[3 + v];
    A.L[3 * (nx - 1) + v] = A.L[3 * (nx - 2) + v];
  }
  __syncthreads();
}

// L(d) into A.L; face fluxes staged in A.fh.  Called by all threads of the CTA.
__device__ void rhs(const Fv1dArgs &A, const double *d) {
  if (A.scheme == WB1D_WB1) {
    rhs_wb1(A, d);
    return;
  }
  const int nx = A.nx;
  const double igm1 = 1.0 / (A.gamma - 1.0);
  for (int f = threadIdx.x; f <= nx; f += blockDim.x) {
    double ue[3] = {A.ref[f], 0.0, A.pef[f] * igm1}, uL[3], uR[3], fl[3], fr[3], fe[3];
    const int il = map1(f - 1, nx, A.bc), ir = map1(f, nx, A.bc);
    for (int v = 0; v < 3; ++v) {
      uL[v] = ue[v] + (d[3 * il + v] + 0.5 * slope(A, d, f - 1, v));
      uR[v] = ue[v] + (d[3 * ir + v] - 0.5 * slope(A, d, f, v));
    }
    flux1(A.gamma, uL, fl);
    flux1(A.gamma, uR, fr);
    flux1(A.gamma, ue, fe);
    double cmax = fmax(speed1(A.gamma, uL), speed1(A.gamma, uR));
    for (int v = 0; v < 3; ++v)
      A.fh[3 * f + v] = (0.5 * (fr[v] + fl[v]) - 0.5 * cmax * (uR[v] - uL[v])) - fe[v];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    double r = A.re[i] + d[3 * i];
    double s[3] = {0.0, -(r * A.g) - (-(A.re[i] * A.g)), -(d[3 * i + 1] * A.g)};
    for (int v = 0; v < 3; ++v) A.L[3 * i + v] = -(A.fh[3 * (i + 1) + v] - A.fh[3 * i + v]) / A.dx + s[v];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(1024) k_fv1d_run(const __grid_constant__ Fv1dArgs A) {
  __shared__ double red[32];
  __shared__ double sdt;
  const int nx = A.nx, tid = threadIdx.x;
  const double igm1 = 1.0 / (A.gamma - 1.0);
  if (A.rhs_only) {
    rhs(A, A.d);
    return;
  }
  double t = *A.t;
  int it = 0;
  while (t < A.tend && it < A.max_steps) {
    // CFL: dt = cfl dx / max(|u| + c) over cell centres
    double cm = 0.0;
    for (int i = tid; i < nx; i += blockDim.x) {
      double u[3] = {A.re[i] + A.d[3 * i], A.d[3 * i + 1], A.pe[i] * igm1 + A.d[3 * i + 2]};
      cm = fmax(cm, speed1(A.gamma, u));
    }
    for (int o = 16; o > 0; o >>= 1) cm = fmax(cm, __shfl_xor_sync(0xffffffffu, cm, o));
    if ((tid & 31) == 0) red[tid >> 5] = cm;
    __syncthreads();
    if (tid == 0) {
      double m = 0.0;
      for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) m = fmax(m, red[w]);
      double dt = A.cfl * A.dx / m;
      if (dt > A.tend - t) dt = A.tend - t;
      sdt = dt;
    }
    __syncthreads();
    const double dt = sdt;
    rhs(A, A.d);
    for (int e = tid; e < 3 * nx; e += blockDim.x) A.w1[e] = A.d[e] + dt * A.L[e];
    __syncthreads();
    rhs(A, A.w1);
    for (int e = tid; e < 3 * nx; e += blockDim.x)
      A.d[e] = 0.5 * A.d[e] + 0.5 * A.w1[e] + 0.5 * dt * A.L[e];
    __syncthreads();
    t += dt;
    ++it;
  }
  if (tid == 0) {
    *A.t = t;
    *A.steps = it;
  }
}

}  // namespace

struct wb1d_ctx {
  wb1d_config cfg;
  double *d = nullptr, *w1 = nullptr, *fh = nullptr, *L = nullptr;
  double *re = nullptr, *pe = nullptr, *ref = nullptr, *pef = nullptr;
  double *t = nullptr;
  int *steps = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
};

namespace {
int e1(wb1d_ctx *c, int code, const std::string &m) {
  if (c) c->err = m;
  return code;
}
#define CK1(call)                                                                       \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return e1(c, WB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

Fv1dArgs args1(wb1d_ctx *c) {
  Fv1dArgs A;
  std::memset(&A, 0, sizeof(A));
  A.nx = c->cfg.nx;
  A.bc = c->cfg.bc;
  A.limiter = c->cfg.limiter;
  A.scheme = c->cfg.scheme;
  A.dx = c->cfg.lx / (double)c->cfg.nx;
  A.gamma = c->cfg.gamma;
  A.g = c->cfg.g;
  A.cfl = c->cfg.cfl;
  A.d = c->d;
  A.w1 = c->w1;
  A.fh = c->fh;
  A.L = c->L;
  A.re = c->re;
  A.pe = c->pe;
  A.ref = c->ref;
  A.pef = c->pef;
  A.t = c->t;
  A.steps = c->steps;
  return A;
}
int threads1(int nx) {
  int t = 32;
  while (t < nx && t < 1024) t *= 2;
  return t;
}
}  // namespace

extern "C" {

const char *wb1d_last_error(const wb1d_ctx *c) { return c ? c->err.c_str() : "null context"; }

int wb1d_destroy(wb1d_ctx *c) {
  if (!c) return WB_OK;
  cudaSetDevice(c->cfg.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  double *bufs[] = {c->d, c->w1, c->fh, c->L, c->re, c->pe, c->ref, c->pef, c->t};
  for (double *b : bufs) cudaFree(b);
  cudaFree(c->steps);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return WB_OK;
}

int wb1d_create(const wb1d_config *cfg, wb1d_ctx **out) {
  if (!cfg || !out) return WB_ERR_ARG;
  wb1d_ctx *c = new wb1d_ctx();
  c->cfg = *cfg;
  *out = c;
  if (cfg->nx < 2 || cfg->nx > (1 << 24)) return e1(c, WB_ERR_CONFIG, "nx must be in [2, 2^24]");
  if (cfg->bc != WB_BC_PERIODIC && cfg->bc != WB_BC_COPY) return e1(c, WB_ERR_CONFIG, "bad bc");
  if (cfg->scheme != WB1D_EQL && cfg->scheme != WB1D_WB1)
    return e1(c, WB_ERR_CONFIG, "scheme must be WB1D_EQL or WB1D_WB1");
  if (cfg->scheme == WB1D_WB1 && cfg->nx < 3) return e1(c, WB_ERR_CONFIG, "'WB1' needs nx >= 3");
  if (cfg->eq_kind != WB_EQ_ISOTHERMAL && cfg->eq_kind != WB_EQ_POLYTROPE)
    return e1(c, WB_ERR_CONFIG, "eq_kind must be isothermal or polytrope");
  if (!(cfg->gamma > 1.0) || !(cfg->lx > 0.0) || !(cfg->cfl > 0.0))
    return e1(c, WB_ERR_CONFIG, "gamma > 1, lx > 0, cfl > 0 required");
  if (cfg->eq_kind == WB_EQ_ISOTHERMAL && !(cfg->rho0 > 0.0 && cfg->p0 > 0.0))
    return e1(c, WB_ERR_CONFIG, "isothermal rho0, p0 must be > 0");
  if (cfg->eq_kind == WB_EQ_POLYTROPE &&
      !(cfg->kpoly > 0.0 && 1.0 - (cfg->gamma - 1.0) / (cfg->gamma * cfg->kpoly) * std::fmax(0.0, cfg->g * cfg->lx) > 0.0))
    return e1(c, WB_ERR_CONFIG, "polytrope density vanishes inside the domain");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return e1(c, WB_ERR_CUDA, "no CUDA device");
  }
  if (cfg->device < 0 || cfg->device >= ndev) return e1(c, WB_ERR_CONFIG, "bad device ordinal");
  CK1(cudaSetDevice(cfg->device));
  CK1(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  const int nx = cfg->nx;
  CK1(cudaMalloc(&c->d, sizeof(double) * 3 * nx));
  CK1(cudaMalloc(&c->w1, sizeof(double) * 3 * nx));
  CK1(cudaMalloc(&c->L, sizeof(double) * 3 * nx));
  CK1(cudaMalloc(&c->fh, sizeof(double) * 3 * (nx + 1)));
  CK1(cudaMalloc(&c->re, sizeof(double) * nx));
  CK1(cudaMalloc(&c->pe, sizeof(double) * nx));
  CK1(cudaMalloc(&c->ref, sizeof(double) * (nx + 1)));
  CK1(cudaMalloc(&c->pef, sizeof(double) * (nx + 1)));
  CK1(cudaMalloc(&c->t, sizeof(double)));
  CK1(cudaMalloc(&c->steps, sizeof(int)));
  // equilibrium at centres and faces: the same separable factors as the 2D path with
  // the potential Phi = g x
  wb::EqParams ep{cfg->eq_kind, cfg->gamma, cfg->g, 0.0, cfg->rho0, cfg->p0, cfg->kpoly};
  const double dx = cfg->lx / (double)nx, fy = wb::eq_factor_y(ep, 0.0);
  std::vector<double> re(nx), pe(nx), ref(nx + 1), pef(nx + 1);
  for (int i = 0; i < nx; ++i) wb::eq_combine(ep, wb::eq_factor_x(ep, ((double)i + 0.5) * dx), fy, &re[i], &pe[i]);
  for (int f = 0; f <= nx; ++f) wb::eq_combine(ep, wb::eq_factor_x(ep, (double)f * dx), fy, &ref[f], &pef[f]);
  CK1(cudaMemcpy(c->re, re.data(), sizeof(double) * nx, cudaMemcpyHostToDevice));
  CK1(cudaMemcpy(c->pe, pe.data(), sizeof(double) * nx, cudaMemcpyHostToDevice));
  CK1(cudaMemcpy(c->ref, ref.data(), sizeof(double) * (nx + 1), cudaMemcpyHostToDevice));
  CK1(cudaMemcpy(c->pef, pef.data(), sizeof(double) * (nx + 1), cudaMemcpyHostToDevice));
  CK1(cudaMemset(c->d, 0, sizeof(double) * 3 * nx));
  CK1(cudaMemset(c->t, 0, sizeof(double)));
  return WB_OK;
}

int wb1d_upload(wb1d_ctx *c, const double *delta) {
  if (!c || !delta) return WB_ERR_ARG;
  CK1(cudaSetDevice(c->cfg.device));
  CK1(cudaMemcpyAsync(c->d, delta, sizeof(double) * 3 * c->cfg.nx, cudaMemcpyHostToDevice, c->stream));
  CK1(cudaMemsetAsync(c->t, 0, sizeof(double), c->stream));
  CK1(cudaStreamSynchronize(c->stream));
  return WB_OK;
}

int wb1d_download(wb1d_ctx *c, double *delta) {
  if (!c || !delta) return WB_ERR_ARG;
  CK1(cudaSetDevice(c->cfg.device));
  CK1(cudaMemcpyAsync(delta, c->d, sizeof(double) * 3 * c->cfg.nx, cudaMemcpyDeviceToHost, c->stream));
  CK1(cudaStreamSynchronize(c->stream));
  return WB_OK;
}

int wb1d_compute_update(wb1d_ctx *c, const double *delta, double *dudt) {
  if (!c || !delta || !dudt) return WB_ERR_ARG;
  CK1(cudaSetDevice(c->cfg.device));
  const int nx = c->cfg.nx;
  CK1(cudaMemcpyAsync(c->w1, delta, sizeof(double) * 3 * nx, cudaMemcpyHostToDevice, c->stream));
  Fv1dArgs A = args1(c);
  A.d = c->w1;
  A.rhs_only = 1;
  k_fv1d_run<<<1, threads1(nx), 0, c->stream>>>(A);
  CK1(cudaGetLastError());
  CK1(cudaMemcpyAsync(dudt, c->L, sizeof(double) * 3 * nx, cudaMemcpyDeviceToHost, c->stream));
  CK1(cudaStreamSynchronize(c->stream));
  return WB_OK;
}

int wb1d_evolve(wb1d_ctx *c, double tend, int32_t max_steps, int32_t *steps_done, double *t_out) {
  if (!c || max_steps < 0) return WB_ERR_ARG;
  CK1(cudaSetDevice(c->cfg.device));
  Fv1dArgs A = args1(c);
  A.tend = tend;
  A.max_steps = max_steps;
  k_fv1d_run<<<1, threads1(c->cfg.nx), 0, c->stream>>>(A);
  CK1(cudaGetLastError());
  double t = 0.0;
  int n = 0;
  CK1(cudaMemcpyAsync(&t, c->t, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK1(cudaMemcpyAsync(&n, c->steps, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK1(cudaStreamSynchronize(c->stream));
  if (steps_done) *steps_done = n;
  if (t_out) *t_out = t;
  if (!std::isfinite(t)) return e1(c, WB_ERR_NONPHYSICAL, "non-finite time step");
  return WB_OK;
}

int wb1d_write_dat(wb1d_ctx *c, const char *path, int32_t var) {
  if (!c || !path || var < 1 || var > 3) return WB_ERR_ARG;
  const int nx = c->cfg.nx;
  std::vector<double> d((size_t)3 * nx);
  int rc = wb1d_download(c, d.data());
  if (rc) return rc;
  wb::EqParams ep{c->cfg.eq_kind, c->cfg.gamma, c->cfg.g, 0.0, c->cfg.rho0, c->cfg.p0, c->cfg.kpoly};
  const double dx = c->cfg.lx / (double)nx, gm1 = c->cfg.gamma - 1.0, fy = wb::eq_factor_y(ep, 0.0);
  FILE *f = std::fopen(path, "w");
  if (!f) return e1(c, WB_ERR_ARG, std::string("cannot open ") + path);
  char num[16];
  for (int i = 0; i < nx; ++i) {
    // primitive state of the full cell value u_eq + delta minus the equilibrium's
    // primitives at the centre: (rho - rho_eq, u, p - p_eq)
    const double x = ((double)i + 0.5) * dx;
    double re, pe;
    wb::eq_combine(ep, wb::eq_factor_x(ep, x), fy, &re, &pe);
    const double *u = &d[(size_t)i * 3];
    const double rho = re + u[0], v = u[1] / rho;
    // the pressure difference without the cancellation p(u_eq + d) - p_eq
    const double w[3] = {u[0], v, gm1 * (u[2] - 0.5 * rho * v * v)};
    wb::fortran_1pe12_5(x, num);  // fields separated by the format's 1X, none trailing
    std::fprintf(f, "%s", num);
    for (int k = var - 1; k < 3; ++k) {
      wb::fortran_1pe12_5(w[k], num);
      std::fprintf(f, " %s", num);
    }
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return WB_OK;
}

}  // extern "C"
