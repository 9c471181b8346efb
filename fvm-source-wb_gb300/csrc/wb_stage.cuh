// wb_stage.cuh -- fused well-balanced modal-DG Runge-Kutta stage for sm_103a.
//
// One CTA owns a TX x TY tile of cells.  Per stage it
//   1. stages the perturbation modes of the tile plus a one-cell halo in shared memory
//      (and, when the limiter is on, the cell means of a two-cell halo);
//   2. applies the minmod moment limiter to every staged cell (limit-on-load: stage
//      outputs are stored unlimited and every consumer limits what it reads, which is
//      the same as the reference's apply_limiter after each stage);
//   3. computes every x- and y-face flux of the tile once (LLF on equilibrium face
//      state + perturbation traces, minus the equilibrium flux);
//   4. per cell: volume and source quadrature of the split fluxes, edge integrals,
//      assembly, the RK stage combination, and (last stage) the CFL wave-speed maxima.
// The reference computes the same quantities in separate whole-array passes
// (2d/benchmark_2d_dg.f90:1137-1479 for the operator, :666-747 for the stage loop,
// :826-870 for the wave speed).
//
// Two arithmetic forms share the code:
//   double  -- "plain": literal split F(u_eq + d) - F(u_eq) at every point
//              (dg_with_source.f90:1749-2031 applied pointwise);
//   float   -- "perturbation": exact difference algebra for zero equilibrium
//              velocity, so a zero perturbation gives an exactly zero update and
//              no O(1) equilibrium quantity is ever subtracted in FP32.
//
// This header is included by one translation unit per precision after it has defined
//   __constant__ wb::Tab1D<R> c_tab[KMAX+1];
#pragma once
#include <type_traits>
#include "wb_types.h"

namespace wb {

__device__ __forceinline__ int wrap_index(int i, int n, int bc) {
  if (i >= 0 && i < n) return i;
  if (bc == 0) {
    int r = i % n;
    return r < 0 ? r + n : r;
  }
  return i < 0 ? 0 : n - 1;
}

template <typename R>
__device__ __forceinline__ R rfmax(R a, R b) { return a > b ? a : b; }

// minmod / generalized minmod of 2d/limiters.f90:18-54
template <typename R>
__device__ __forceinline__ R minmod3(R x, R y, R z) {
  R s = copysign(R(1), x);
  if (copysign(R(1), y) == s && copysign(R(1), z) == s) return s * fmin(fmin(fabs(x), fabs(y)), fabs(z));
  return R(0);
}
template <typename R>
__device__ __forceinline__ R gminmod(R x, R y, R z, R Mh2) {
  if (fabs(x) < Mh2) return x;
  return minmod3(x, y, z);
}

// Equilibrium density/pressure from the separable factors (see wb_tables.cpp).
template <typename R>
__device__ __forceinline__ void eq_point(const StageArgs<R> &A, R fx, R fy, R &re, R &pe) {
  if (A.eq_kind == 1) {
    R t = fx * fy;
    re = A.rho0 * t;
    pe = A.p0 * t;
  } else if (A.eq_kind == 2) {
    R s = fx + fy;
    re = pow(s, A.npoly);
    pe = A.kpoly * (re * s);
  } else {
    re = R(0);
    pe = R(0);
  }
}

// ---------------------------------------------------------------- FP64 literal
// compute_primitive / compute_flux_int / get_source of 2d/benchmark_2d_dg.f90:891-963
// and benchmark_2d.f90:327-350.
__device__ __forceinline__ void prim_lit(const double *u, double *w, double gm1) {
  w[0] = fmax(u[0], (double)1.0e-9f);
  double inv = 1.0 / w[0];
  w[1] = u[1] * inv;
  w[2] = u[2] * inv;
  w[3] = gm1 * (u[3] - 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2]));
}
template <int DIR>
__device__ __forceinline__ void flux_lit(const double *u, const double *w, double *f) {
  if (DIR == 0) {
    f[0] = w[1] * u[0];
    f[1] = w[1] * u[1] + w[3];
    f[2] = w[0] * w[1] * w[2];
    f[3] = w[1] * u[3] + w[1] * w[3];
  } else {
    f[0] = w[2] * u[0];
    f[1] = w[0] * w[1] * w[2];
    f[2] = w[2] * u[2] + w[3];
    f[3] = w[2] * u[3] + w[2] * w[3];
  }
}

// Volume point: split fluxes and source, already scaled by 0.5/dx, 0.5/dy, 0.25.
template <typename R>
__device__ __forceinline__ void vol_point(const StageArgs<R> &A, const R *d, R re, R pe, R *Fx,
                                          R *Fy, R *S) {
  if constexpr (std::is_same<R, double>::value) {
    double ue[NV] = {re, 0.0, 0.0, pe * A.igm1}, u[NV], w[NV], we[NV], f[NV], fe[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) u[v] = ue[v] + d[v];
    prim_lit(u, w, A.gm1);
    prim_lit(ue, we, A.gm1);
    flux_lit<0>(u, w, f);
    flux_lit<0>(ue, we, fe);
#pragma unroll
    for (int v = 0; v < NV; ++v) Fx[v] = (f[v] - fe[v]) * A.hidx;
    flux_lit<1>(u, w, f);
    flux_lit<1>(ue, we, fe);
#pragma unroll
    for (int v = 0; v < NV; ++v) Fy[v] = (f[v] - fe[v]) * A.hidy;
    double s[NV], se[NV];
    s[0] = 0.0;
    s[1] = -(w[0] * A.gx);
    s[2] = -(w[0] * A.gy);
    s[3] = -(w[0] * (w[1] * A.gx + w[2] * A.gy));
    se[0] = 0.0;
    se[1] = -(we[0] * A.gx);
    se[2] = -(we[0] * A.gy);
    se[3] = -(we[0] * (we[1] * A.gx + we[2] * A.gy));
#pragma unroll
    for (int v = 0; v < NV; ++v) S[v] = (s[v] - se[v]) * 0.25;
  } else {
    // exact differences about a static equilibrium (u_eq velocity 0):
    //   d(rho u) = m_x, d(rho u^2 + p) = m_x^2/rho + dp, d(rho u v) = m_x m_y / rho,
    //   d(u (E+p)) = u (H_eq + dE + dp), dp = (gamma-1)(dE - |m|^2/(2 rho)),
    //   dS = (0, -drho gx, -drho gy, -(m_x gx + m_y gy))
    R r = rfmax(re + d[0], R(1.0e-9f));
    R inv = R(1) / r;
    R vx = d[1] * inv, vy = d[2] * inv;
    R dp = A.gm1 * (d[3] - R(0.5) * (d[1] * vx + d[2] * vy));
    R H = A.hgam * pe + d[3] + dp;
    Fx[0] = d[1] * A.hidx;
    Fx[1] = (d[1] * vx + dp) * A.hidx;
    Fx[2] = (d[2] * vx) * A.hidx;
    Fx[3] = (vx * H) * A.hidx;
    Fy[0] = d[2] * A.hidy;
    Fy[1] = (d[1] * vy) * A.hidy;
    Fy[2] = (d[2] * vy + dp) * A.hidy;
    Fy[3] = (vy * H) * A.hidy;
    S[0] = R(0);
    S[1] = -(d[0] * A.gx) * R(0.25);
    S[2] = -(d[0] * A.gy) * R(0.25);
    S[3] = -(d[1] * A.gx + d[2] * A.gy) * R(0.25);
  }
}

// Face point in direction DIR: LLF flux difference (F_hat - F(u_eq)) from perturbation
// traces dL (left/bottom) and dR (right/top) on the equilibrium face state.
// compute_llflux, 2d/benchmark_2d_dg.f90:968-988.
template <typename R, int DIR>
__device__ __forceinline__ void face_point(const StageArgs<R> &A, const R *dL, const R *dR, R re,
                                           R pe, R *F) {
  if constexpr (std::is_same<R, double>::value) {
    double ue[NV] = {re, 0.0, 0.0, pe * A.igm1}, uL[NV], uR[NV], wL[NV], wR[NV], we[NV];
    double fL[NV], fR[NV], fe[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      uL[v] = ue[v] + dL[v];
      uR[v] = ue[v] + dR[v];
    }
    prim_lit(uL, wL, A.gm1);
    prim_lit(uR, wR, A.gm1);
    prim_lit(ue, we, A.gm1);
    flux_lit<DIR>(uL, wL, fL);
    flux_lit<DIR>(uR, wR, fR);
    flux_lit<DIR>(ue, we, fe);
    double cL = sqrt(A.gamma * fmax(wL[3], 1e-10) / fmax(wL[0], 1e-10));
    double cR = sqrt(A.gamma * fmax(wR[3], 1e-10) / fmax(wR[0], 1e-10));
    double vL = wL[1 + DIR], vR = wR[1 + DIR], lam;
    if (A.llf_speed == 1)
      lam = fmax(fabs(vR + cR), fabs(vL + cL));
    else
      lam = fmax(fabs(vL) + cL, fabs(vR) + cR);
#pragma unroll
    for (int v = 0; v < NV; ++v) F[v] = (0.5 * (fR[v] + fL[v]) + 0.5 * lam * (uL[v] - uR[v])) - fe[v];
  } else {
    R fL[NV], fR[NV], lamL, lamR;
    R hp = A.hgam * pe;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const R *d = s == 0 ? dL : dR;
      R *f = s == 0 ? fL : fR;
      R r = rfmax(re + d[0], R(1.0e-9f));
      R inv = R(1) / r;
      R vx = d[1] * inv, vy = d[2] * inv;
      R dp = A.gm1 * (d[3] - R(0.5) * (d[1] * vx + d[2] * vy));
      R H = hp + d[3] + dp;
      R vn = DIR == 0 ? vx : vy;
      f[0] = d[1 + DIR];
      f[1] = DIR == 0 ? d[1] * vx + dp : d[1] * vy;
      f[2] = DIR == 0 ? d[2] * vx : d[2] * vy + dp;
      f[3] = vn * H;
      R c = sqrt(A.gamma * rfmax(pe + dp, R(1e-10)) * inv);
      R lam = A.llf_speed == 1 ? vn + c : fabs(vn) + c;
      if (s == 0) lamL = lam; else lamR = lam;
    }
    R lam = A.llf_speed == 1 ? rfmax(fabs(lamR), fabs(lamL)) : rfmax(lamL, lamR);
#pragma unroll
    for (int v = 0; v < NV; ++v) F[v] = R(0.5) * (fR[v] + fL[v]) + R(0.5) * lam * (dL[v] - dR[v]);
  }
}

// Limit one cell's modes in place (base[m*mstride] is mode m of one variable).
template <typename R, int K, int BASIS>
__device__ __forceinline__ void limit_modes(const StageArgs<R> &A, R *base, int mstride, R m0,
                                            R mw, R me, R ms, R mn) {
  if constexpr (K >= 1) {
    constexpr int NB = num_modes(K, BASIS);
    constexpr int M10 = mode_index(K, BASIS, 1, 0), M01 = mode_index(K, BASIS, 0, 1);
    R sx = base[M10 * mstride], sy = base[M01 * mstride];
    R l1 = gminmod(A.lim_norm * sx, me - m0, m0 - mw, A.lim_Mdx2) / A.lim_norm;
    R l2 = gminmod(A.lim_norm * sy, mn - m0, m0 - ms, A.lim_Mdy2) / A.lim_norm;
    if (fabs(l1 - sx) > A.lim_tol || fabs(l2 - sy) > A.lim_tol) {
      base[M10 * mstride] = l1;
      base[M01 * mstride] = l2;
#pragma unroll
      for (int m = 0; m < NB; ++m)
        if (mode_deg(K, BASIS, m, 0) + mode_deg(K, BASIS, m, 1) >= 2) base[m * mstride] = R(0);
    }
  }
}

__device__ __forceinline__ double block_max(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  int nthr = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
  int warp = tid >> 5, lane = tid & 31;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (nthr + 31) / 32 ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  __syncthreads();
  return v;
}

template <typename R>
__device__ __forceinline__ double stage_dt(const StageArgs<R> &A) {
  if (A.dt_mode == 0) return A.dt_fixed;
  const DevState *S = A.dev;
  double sx = __longlong_as_double((long long)S->smax[A.parity][0]);
  double sy = __longlong_as_double((long long)S->smax[A.parity][1]);
  double dt = A.cfl_over / (sx / A.ddx + sy / A.ddy);
  if (A.tend > 0.0) {
    double rem = A.tend - S->t[A.parity];
    dt = rem <= 0.0 ? 0.0 : fmin(dt, rem);
  }
  return dt;
}

// Shared-memory bytes for a TX x TY tile.
template <typename R>
__host__ __device__ inline size_t stage_smem_bytes(int K, int basis, int TX, int TY, int lim) {
  int NB = num_modes(K, basis), NQ = K + 1;
  size_t n = (size_t)NV * NB * (TY + 2) * (TX + 2);
  if (lim) n += (size_t)NV * (TY + 4) * (TX + 4);
  n += (size_t)NV * NQ * TY * (TX + 1) + (size_t)NV * NQ * (TY + 1) * TX;
  return n * sizeof(R) + 64 * sizeof(double);
}

template <typename R, int K, int BASIS>
__global__ void __launch_bounds__(256, std::is_same<R, float>::value ? 2 : 1)
    k_stage(const __grid_constant__ StageArgs<R> A) {
  constexpr int NQ = K + 1;
  constexpr int NB = num_modes(K, BASIS);
  const Tab1D<R> &T = c_tab[K];
  const int TX = blockDim.x, TY = blockDim.y;
  const int RX = TX + 2, RY = TY + 2, RXY = RX * RY;
  const int LX = TX + 4, LY = TY + 4;
  const int tid = threadIdx.y * TX + threadIdx.x, nthr = TX * TY;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int nx = A.nx, ny = A.ny;
  const long long P = A.plane;
  const bool lim = A.limiter && A.lim_y && K >= 1;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *red = reinterpret_cast<double *>(smem_raw);
  R *su = reinterpret_cast<R *>(smem_raw + 64 * sizeof(double));
  R *sm = su + NV * NB * RXY;
  R *sfx = sm + (lim ? NV * LY * LX : 0);
  const int FXS = TY * (TX + 1);
  R *sfy = sfx + NV * NQ * FXS;
  const int FYS = (TY + 1) * TX;

  const double dt = stage_dt(A);
  if (A.advance_time && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) {
    DevState *S = A.dev;
    S->t[A.parity ^ 1] = S->t[A.parity] + dt;
    S->nstep[A.parity ^ 1] = S->nstep[A.parity] + 1;
    S->smax[A.parity ^ 1][0] = 0ull;
    S->smax[A.parity ^ 1][1] = 0ull;
  }

  // 1. stage modes of the tile + one-cell halo (BC-mapped), and halo-2 means
  for (int e = tid; e < NV * NB * RXY; e += nthr) {
    int rx = e % RX, t1 = e / RX, ry = t1 % RY, pl = t1 / RY;
    int gi = wrap_index(i0 + rx - 1, nx, A.bc_x), gj = wrap_index(j0 + ry - 1, ny, A.bc_y);
    su[e] = A.x[pl * P + (long long)gj * nx + gi];
  }
  if (lim) {
    for (int e = tid; e < NV * LY * LX; e += nthr) {
      int lx = e % LX, t1 = e / LX, ly = t1 % LY, v = t1 / LY;
      int gi = wrap_index(i0 + lx - 2, nx, A.bc_x), gj = wrap_index(j0 + ly - 2, ny, A.bc_y);
      sm[e] = A.x[(long long)(v * NB) * P + (long long)gj * nx + gi];
    }
  }
  __syncthreads();

  // 2. limiter on every staged cell (means never change, so cells are independent)
  if (lim) {
    for (int e = tid; e < NV * RXY; e += nthr) {
      int rx = e % RX, t1 = e / RX, ry = t1 % RY, v = t1 / RY;
      const R *mv = sm + v * LY * LX;
      int c = (ry + 1) * LX + (rx + 1);
      limit_modes<R, K, BASIS>(A, su + (v * NB) * RXY + ry * RX + rx, RXY, mv[c], mv[c - 1],
                               mv[c + 1], mv[c - LX], mv[c + LX]);
    }
    __syncthreads();
  }

  // 3a. x faces: (TX+1) x TY, face fi sits between tile cells fi-1 and fi
  for (int f = tid; f < FXS; f += nthr) {
    int fi = f % (TX + 1), fj = f / (TX + 1);
    int gfi = i0 + fi, gj = j0 + fj;
    if (gfi > nx || gj >= ny) continue;
    R cl[NV][NQ], cr[NV][NQ];
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int b = 0; b < NQ; ++b) {
        R sl = R(0), sr = R(0);
#pragma unroll
        for (int a = 0; a < NQ; ++a) {
          constexpr int dummy = 0;
          (void)dummy;
          int m = mode_index(K, BASIS, a, b);
          if (m < 0) continue;
          const R *pm = su + (v * NB + m) * RXY + (fj + 1) * RX;
          sl += pm[fi] * T.Ep[a];
          sr += pm[fi + 1] * T.Em[a];
        }
        cl[v][b] = sl;
        cr[v][b] = sr;
      }
    const R fxf = A.fxf[gfi];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      R dL[NV], dR[NV], F[NV], re, pe;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        R sl = R(0), sr = R(0);
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          sl += cl[v][b] * T.B[b][q];
          sr += cr[v][b] * T.B[b][q];
        }
        dL[v] = sl;
        dR[v] = sr;
      }
      eq_point(A, fxf, A.fyv[gj * NQ + q], re, pe);
      face_point<R, 0>(A, dL, dR, re, pe, F);
#pragma unroll
      for (int v = 0; v < NV; ++v) sfx[(v * NQ + q) * FXS + f] = F[v];
    }
  }
  // 3b. y faces: TX x (TY+1), face fj sits between tile cells fj-1 and fj
  for (int f = tid; f < FYS; f += nthr) {
    int fi = f % TX, fj = f / TX;
    int gi = i0 + fi, gfj = j0 + fj;
    if (gi >= nx || gfj > ny) continue;
    R cb[NV][NQ], ct[NV][NQ];
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int a = 0; a < NQ; ++a) {
        R sb = R(0), st = R(0);
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          int m = mode_index(K, BASIS, a, b);
          if (m < 0) continue;
          const R *pm = su + (v * NB + m) * RXY + (fi + 1);
          sb += pm[fj * RX] * T.Ep[b];
          st += pm[(fj + 1) * RX] * T.Em[b];
        }
        cb[v][a] = sb;
        ct[v][a] = st;
      }
    const R fyf = A.fyf[gfj];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      R dB[NV], dT[NV], F[NV], re, pe;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        R sb = R(0), st = R(0);
#pragma unroll
        for (int a = 0; a < NQ; ++a) {
          sb += cb[v][a] * T.B[a][q];
          st += ct[v][a] * T.B[a][q];
        }
        dB[v] = sb;
        dT[v] = st;
      }
      eq_point(A, A.fxv[gi * NQ + q], fyf, re, pe);
      face_point<R, 1>(A, dB, dT, re, pe, F);
#pragma unroll
      for (int v = 0; v < NV; ++v) sfy[(v * NQ + q) * FYS + f] = F[v];
    }
  }
  __syncthreads();

  // 4. cells
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int gi = i0 + tx, gj = j0 + ty;
  const bool active = gi < nx && gj < ny;
  double spx = 0.0, spy = 0.0;
  if (active) {
    const R *uc = su + (ty + 1) * RX + (tx + 1);  // mode m of var v at uc[(v*NB+m)*RXY]
    R acc[NV][NB];
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int m = 0; m < NB; ++m) acc[v][m] = R(0);
    R rbar = R(0), pbar = R(0);
#pragma unroll
    for (int qa = 0; qa < NQ; ++qa) {
      R c[NV][NQ];
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          R s = R(0);
#pragma unroll
          for (int a = 0; a < NQ; ++a) {
            int m = mode_index(K, BASIS, a, b);
            if (m < 0) continue;
            s += uc[(v * NB + m) * RXY] * T.B[a][qa];
          }
          c[v][b] = s;
        }
      const R fx = A.fxv[gi * NQ + qa];
      R Pq[NV][NQ], Qq[NV][NQ];
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int b = 0; b < NQ; ++b) Pq[v][b] = Qq[v][b] = R(0);
#pragma unroll
      for (int qb = 0; qb < NQ; ++qb) {
        R d[NV], Fx[NV], Fy[NV], S[NV], re, pe;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          R s = R(0);
#pragma unroll
          for (int b = 0; b < NQ; ++b) s += c[v][b] * T.B[b][qb];
          d[v] = s;
        }
        eq_point(A, fx, A.fyv[gj * NQ + qb], re, pe);
        if (A.compute_speed) {
          R ww = R(0.25) * T.wq[qa] * T.wq[qb];
          rbar += re * ww;
          pbar += pe * ww;
        }
        vol_point(A, d, re, pe, Fx, Fy, S);
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
          for (int b = 0; b < NQ; ++b) {
            Pq[v][b] += Fx[v] * T.BW[b][qb];
            Qq[v][b] += S[v] * T.BW[b][qb];
            if (b > 0) Qq[v][b] += Fy[v] * T.DW[b][qb];
          }
      }
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int m = 0; m < NB; ++m) {
          constexpr int dummy = 0;
          (void)dummy;
          int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
          R t = T.BW[a][qa] * Qq[v][b];
          if (a > 0) t += T.DW[a][qa] * Pq[v][b];
          acc[v][m] += t;
        }
    }
    // edge integrals (faces of this cell from shared memory)
    const int fl = ty * (TX + 1) + tx, fb = ty * TX + tx;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      R FR[NQ], FL[NQ], GT[NQ], GB[NQ];
#pragma unroll
      for (int b = 0; b < NQ; ++b) {
        R r = R(0), l = R(0), t = R(0), bt = R(0);
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const R *px = sfx + (v * NQ + q) * FXS;
          const R *py = sfy + (v * NQ + q) * FYS;
          r += px[fl + 1] * T.BW[b][q];
          l += px[fl] * T.BW[b][q];
          t += py[fb + TX] * T.BW[b][q];
          bt += py[fb] * T.BW[b][q];
        }
        FR[b] = r;
        FL[b] = l;
        GT[b] = t;
        GB[b] = bt;
      }
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
        acc[v][m] -= A.hidx * (T.Ep[a] * FR[b] - T.Em[a] * FL[b]) +
                     A.hidy * (T.Ep[b] * GT[a] - T.Em[b] * GB[a]);
      }
    }

    // RK stage combination: out = sum c_i [lim](in_i) + beta Y + (cdt dt) L(Y)
    const long long cell = (long long)gj * nx + gi;
#pragma unroll
    for (int oi = 0; oi < 2; ++oi) {
      const Combo<R> &o = A.o[oi];
      if (o.out == nullptr) continue;
      R val[NV][NB];
      const R cdt = o.cdt * (R)dt;
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int m = 0; m < NB; ++m) val[v][m] = R(0);
#pragma unroll
      for (int ii = 0; ii < 2; ++ii) {
        if (o.in[ii] == nullptr) continue;
        const R *in = o.in[ii];
        R w[NV][NB];
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
          for (int m = 0; m < NB; ++m) w[v][m] = in[(long long)(v * NB + m) * P + cell];
        if (o.lim[ii] && A.limiter && K >= 1) {
          int iw = wrap_index(gi - 1, nx, A.bc_x), ie = wrap_index(gi + 1, nx, A.bc_x);
          int js = wrap_index(gj - 1, ny, A.bc_y), jn = wrap_index(gj + 1, ny, A.bc_y);
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const R *m0p = in + (long long)(v * NB) * P;
            limit_modes<R, K, BASIS>(A, &w[v][0], 1, w[v][0], m0p[(long long)gj * nx + iw],
                                     m0p[(long long)gj * nx + ie], m0p[(long long)js * nx + gi],
                                     m0p[(long long)jn * nx + gi]);
          }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
          for (int m = 0; m < NB; ++m) val[v][m] += o.c[ii] * w[v][m];
      }
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int m = 0; m < NB; ++m) {
          R y = uc[(v * NB + m) * RXY];
          R r = (val[v][m] + o.beta * y) + cdt * acc[v][m];
          o.out[(long long)(v * NB + m) * P + cell] = r;
          if (oi == 0) val[v][m] = r;  // keep o[0]'s means for the wave speed
        }
      if (oi == 0 && A.compute_speed) {
        // wave speed from the new cell mean of the full state
        R d0 = val[0][0], d1 = val[1][0], d2 = val[2][0], d3 = val[3][0];
        R r = rbar + d0;
        R rf = rfmax(r, R(1.0e-9f));
        R inv = R(1) / rf;
        R vx = d1 * inv, vy = d2 * inv;
        R p;
        if constexpr (std::is_same<R, double>::value)
          p = A.gm1 * ((pbar * A.igm1 + d3) - R(0.5) * rf * (vx * vx + vy * vy));
        else
          p = pbar + A.gm1 * (d3 - R(0.5) * (d1 * vx + d2 * vy));
        R cs = sqrt(A.gamma * rfmax(p, R(1e-10)) / rfmax(rf, R(1e-10)));
        spx = (double)(fabs(vx) + cs);
        spy = (double)(fabs(vy) + cs);
        bool bad = !(r > R(0)) || !(p > R(0)) || !isfinite(spx) || !isfinite(spy);
        if (A.eq_kind == 0) bad = !isfinite(spx) || !isfinite(spy);
        if (bad) atomicOr(&A.dev->err, 1);
        if (!isfinite(spx)) spx = 0.0;
        if (!isfinite(spy)) spy = 0.0;
      }
    }
  }
  if (A.compute_speed) {
    double mx = block_max(spx, red);
    double my = block_max(spy, red);
    if (tid == 0) {
      atomicMax(&A.dev->smax[A.parity ^ 1][0], (unsigned long long)__double_as_longlong(mx));
      atomicMax(&A.dev->smax[A.parity ^ 1][1], (unsigned long long)__double_as_longlong(my));
    }
  }
}

}  // namespace wb
