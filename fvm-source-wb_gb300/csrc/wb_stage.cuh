// wb_stage.cuh -- fused well-balanced modal-DG Runge-Kutta stage for sm_103a.
//
// One CTA owns a TX x TY tile of cells.  Per stage it
//   1. stages the perturbation modes of the tile plus a one-cell halo in shared memory
//      (and, when the limiter is on, the cell means of a two-cell halo);
//   2. applies the limiter to every staged cell -- the minmod moment limiter or the
//      Zhang-Shu positivity limiter (limit-on-load: stage outputs are stored unlimited
//      and every consumer limits what it reads, which is the same as the reference's
//      apply_limiter after each stage);
//   3. computes every x- and y-face flux of the tile once (LLF or HLLC on equilibrium
//      face state + perturbation traces, minus the equilibrium flux);
//   4. per cell: volume and source quadrature of the split fluxes, edge integrals,
//      assembly, the RK stage combination, and (last stage) the CFL wave-speed maxima.
//      In FP32 the edge integrals come first; the face-flux area then receives the
//      tile's first RK input by cp.async while the volume quadrature runs.
// Interior tiles of the persistent kernel are staged by one TMA copy, the rest by
// cp.async; the next tile is staged while the current one is computed.
// The reference computes the same quantities in separate whole-array passes
// (2d/benchmark_2d_dg.f90:1137-1479 for the operator, :666-747 for the stage loop,
// :826-870 for the wave speed).
//
// Two arithmetic forms share the code:
//   double  -- "plain": literal split F(u_eq + d) - F(u_eq) at every point
//              (dg_with_source.f90:1749-2031 applied pointwise);
//   float   -- "perturbation": exact difference algebra for zero equilibrium
//              velocity, so a zero perturbation gives an exactly zero update and
//              no O(1) equilibrium quantity is ever subtracted in FP32.  Its volume
//              quadrature and LLF faces run on packed f32x2 pairs (__ffma2_rn and
//              friends), which halves the issue slots of that arithmetic.
//
// The stage kernels read only the compile-time tables of wb_ctab.h; one translation unit
// per compiled instance includes this header (wb_stage_instances.h).
#pragma once
#include <cuda.h>
#include <type_traits>
#include "wb_ctab.h"
#include "wb_types.h"

namespace wb {

// Compile-time basis tables of degree K in the kernel's precision.
template <typename R, int K>
struct TC {
  static __device__ __forceinline__ constexpr R B(int a, int q) { return R(CTab<K>::B(a, q)); }
  static __device__ __forceinline__ constexpr R D(int a, int q) { return R(CTab<K>::D(a, q)); }
  static __device__ __forceinline__ constexpr R BW(int a, int q) { return R(CTab<K>::BW(a, q)); }
  static __device__ __forceinline__ constexpr R DW(int a, int q) { return R(CTab<K>::DW(a, q)); }
  static __device__ __forceinline__ constexpr R Ep(int a) { return R(CTab<K>::Ep(a)); }
  static __device__ __forceinline__ constexpr R Em(int a) { return R(CTab<K>::Em(a)); }
  static __device__ __forceinline__ constexpr R wq(int q) { return R(CTab<K>::wq(q)); }
  static constexpr int NG = CTab<K>::NG;
  static __device__ __forceinline__ constexpr R Gl(int a, int g) { return R(CTab<K>::Gl(a, g)); }
};

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

// Reciprocal and square root of the FP32 perturbation form: the hardware approximations
// (MUFU, about 1 ulp), well inside the form's 1e-6 error budget.  FP64 stays IEEE.
__device__ __forceinline__ float frcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double frcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float fsqrt_pos(float x) { return x * rsqrtf(x); }
__device__ __forceinline__ double fsqrt_pos(double x) { return sqrt(x); }

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

// s^n for the polytropic equilibrium.  FP32 form: the fast intrinsic (MUFU exp2/log2,
// about 1e-7 relative), against an accurate powf that costs tens of instructions at every
// quadrature point.  The equilibrium values enter the FP32 form only as coefficients of
// perturbation terms, so this is far inside its 1e-6 budget; FP64 stays IEEE.
__device__ __forceinline__ float eq_pow(float s, float n) { return __powf(s, n); }
__device__ __forceinline__ double eq_pow(double s, double n) { return pow(s, n); }

// Equilibrium density/pressure from the separable factors (see wb_tables.cpp).
// kind: the instance's equilibrium (its eq_kind); the constants come from A.
template <typename R>
__device__ __forceinline__ void eq_point(const StageArgs<R> &A, const int kind, R fx, R fy, R &re,
                                         R &pe) {
  if (kind == 1) {
    R t = fx * fy;
    re = A.rho0 * t;
    pe = A.p0 * t;
  } else if (kind == 2) {
    R s = fx + fy;
    re = eq_pow(s, A.npoly);
    pe = A.kpoly * (re * s);
  } else {
    re = R(0);
    pe = R(0);
  }
}
template <typename R>
__device__ __forceinline__ void eq_point(const StageArgs<R> &A, R fx, R fy, R &re, R &pe) {
  eq_point(A, A.eq_kind, fx, fy, re, pe);
}

// CFL wave speeds |u| + c and |v| + c of a cell from its mean perturbation d0..d3 and its
// mean equilibrium (rbar, pbar); r and p are the full mean density and pressure.  The one
// formula of the stage kernels' maxima and of the set-up kernels (k_max_speed,
// k_batch_max_speed), so a restart recomputes bit-identical speeds.  FP32 takes the
// hardware reciprocal and square root (about 1 ulp); FP64 stays IEEE.
template <typename R>
__device__ __forceinline__ void mean_wave_speed(const StageArgs<R> &A, R rbar, R pbar, R d0,
                                                R d1, R d2, R d3, R &r, R &p, R &spx, R &spy) {
  r = rbar + d0;
  const R rf = rfmax(r, R(1.0e-9f));
  const R inv = frcp(rf);
  const R vx = d1 * inv, vy = d2 * inv;
  R cs;
  if constexpr (std::is_same<R, double>::value) {
    p = A.gm1 * ((pbar * A.igm1 + d3) - R(0.5) * rf * (vx * vx + vy * vy));
    cs = sqrt(A.gamma * rfmax(p, R(1e-10)) / rfmax(rf, R(1e-10)));
  } else {
    p = pbar + A.gm1 * (d3 - R(0.5) * (d1 * vx + d2 * vy));
    cs = fsqrt_pos(A.gamma * rfmax(p, R(1e-10)) * frcp(rfmax(rf, R(1e-10))));
  }
  spx = fabs(vx) + cs;
  spy = fabs(vy) + cs;
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

// FP64 volume point: split fluxes F(u_eq + d) - F(u_eq) (unscaled) and the source (scaled
// by the 0.25 of the assembly).  The FP32 form evaluates its volume points on packed pairs
// inside tile_compute.
__device__ __forceinline__ void vol_point(const StageArgs<double> &A, const double *d, double re,
                                          double pe, double *Fx, double *Fy, double *S) {
  double ue[NV] = {re, 0.0, 0.0, pe * A.igm1}, u[NV], w[NV], we[NV], f[NV], fe[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) u[v] = ue[v] + d[v];
  prim_lit(u, w, A.gm1);
  prim_lit(ue, we, A.gm1);
  flux_lit<0>(u, w, f);
  flux_lit<0>(ue, we, fe);
#pragma unroll
  for (int v = 0; v < NV; ++v) Fx[v] = f[v] - fe[v];
  flux_lit<1>(u, w, f);
  flux_lit<1>(ue, we, fe);
#pragma unroll
  for (int v = 0; v < NV; ++v) Fy[v] = f[v] - fe[v];
  // rounded products (never contracted into the subtraction below): S(u_eq + 0) and
  // S(u_eq) must round identically so a zero perturbation cancels exactly
  double s[NV], se[NV];
  s[0] = 0.0;
  s[1] = -__dmul_rn(w[0], A.gx);
  s[2] = -__dmul_rn(w[0], A.gy);
  s[3] = -__dmul_rn(w[0], __dadd_rn(__dmul_rn(w[1], A.gx), __dmul_rn(w[2], A.gy)));
  se[0] = 0.0;
  se[1] = -__dmul_rn(we[0], A.gx);
  se[2] = -__dmul_rn(we[0], A.gy);
  se[3] = -__dmul_rn(we[0], __dadd_rn(__dmul_rn(we[1], A.gx), __dmul_rn(we[2], A.gy)));
#pragma unroll
  for (int v = 0; v < NV; ++v) S[v] = (s[v] - se[v]) * 0.25;
}

// Face point in direction DIR: numerical flux minus the equilibrium flux, F_hat - F(u_eq),
// from perturbation traces dL (left/bottom) and dR (right/top) on the equilibrium face
// state.  LLF: compute_llflux, 2d/benchmark_2d_dg.f90:968-988.  HLLC (compile-time switch):
// riemann_hllc, dg_with_source.f90:1318-1374, with Davis wave speeds, the contact speed
// from the Lagrangian sound speeds, the transverse velocity carried by the contact, and
// the star fluxes in the form F_K + S_K (U*_K - U_K),
//   U*_K - U_K = (S* - v_K) / (S_K - S*) [rho_K, rho_K S_K, rho_K vt_K, E_K + p_K + rho_K S* (S_K - v_K)],
// which is riemann_hllc's F(U*_K) in exact arithmetic.  Every star correction carries the
// factor S* - v_K, which is exactly zero for a zero perturbation, so both forms keep the
// equilibrium exactly.
template <typename R, int DIR, bool HLLC>
__device__ __forceinline__ void face_point(const StageArgs<R> &A, const R *dL, const R *dR, R re,
                                           R pe, R *F) {
  constexpr int N = 1 + DIR, T = 2 - DIR;  // normal and transverse momentum
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
    double vL = wL[N], vR = wR[N];
    if constexpr (HLLC) {
      const double SL = fmin(vL, vR) - fmax(cL, cR), SR = fmax(vL, vR) + fmax(cL, cR);
      const double DL = wL[0] * (vL - SL), DR = wR[0] * (SR - vR);
      const double Ss = (DR * vR + DL * vL + (wL[3] - wR[3])) / (DL + DR);
      if (SL > 0.0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) F[v] = fL[v] - fe[v];
      } else if (!(Ss > 0.0) && !(SR > 0.0)) {
#pragma unroll
        for (int v = 0; v < NV; ++v) F[v] = fR[v] - fe[v];
      } else {  // the star regions, sampled in riemann_hllc's order
        const bool left = Ss > 0.0;
        const double *u = left ? uL : uR, *w = left ? wL : wR, *f = left ? fL : fR;
        const double SK = left ? SL : SR, vK = w[N];
        const double q = SK * ((Ss - vK) / (SK - Ss));
        double d[NV];
        d[0] = w[0];
        d[N] = w[0] * SK;
        d[T] = w[0] * w[T];
        d[3] = (u[3] + w[3]) + w[0] * Ss * (SK - vK);
#pragma unroll
        for (int v = 0; v < NV; ++v) F[v] = (f[v] + q * d[v]) - fe[v];
      }
    } else {
      double lam;
      if (A.llf_speed == 1)
        lam = fmax(fabs(vR + cR), fabs(vL + cL));
      else
        lam = fmax(fabs(vL) + cL, fabs(vR) + cR);
#pragma unroll
      for (int v = 0; v < NV; ++v)
        F[v] = (0.5 * (fR[v] + fL[v]) + 0.5 * lam * (uL[v] - uR[v])) - fe[v];
    }
  } else {
    // FP32 (HLLC only: the LLF faces run on packed pairs, face_point_pk).  Exact-difference
    // side quantities: r = rho, vn / vt = normal / transverse velocity, dp = pressure
    // perturbation, H = E + p of the full state, f = flux difference
    static_assert(HLLC, "FP32 LLF faces use face_point_pk");
    R fL[NV], fR[NV], rs[2], vns[2], vts[2], dps[2], Hs[2], cs[2];
    R hp = A.hgam * pe;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const R *d = s == 0 ? dL : dR;
      R *f = s == 0 ? fL : fR;
      R r = rfmax(re + d[0], R(1.0e-9f));
      R inv = frcp(r);
      R vx = d[1] * inv, vy = d[2] * inv;
      R dp = A.gm1 * (d[3] - R(0.5) * (d[1] * vx + d[2] * vy));
      R H = hp + d[3] + dp;
      R vn = DIR == 0 ? vx : vy;
      f[0] = d[1 + DIR];
      f[1] = DIR == 0 ? d[1] * vx + dp : d[1] * vy;
      f[2] = DIR == 0 ? d[2] * vx : d[2] * vy + dp;
      f[3] = vn * H;
      R c = fsqrt_pos(A.gamma * rfmax(pe + dp, R(1e-10)) * inv);
      rs[s] = r;
      vns[s] = vn;
      vts[s] = DIR == 0 ? vy : vx;
      dps[s] = dp;
      Hs[s] = H;
      cs[s] = c;
    }
    {
      const R SL = fmin(vns[0], vns[1]) - fmax(cs[0], cs[1]);
      const R SR = fmax(vns[0], vns[1]) + fmax(cs[0], cs[1]);
      const R DL = rs[0] * (vns[0] - SL), DR = rs[1] * (SR - vns[1]);
      // p_L - p_R = dp_L - dp_R: the equilibrium pressure is the same on both sides
      const R Ss = (DR * vns[1] + DL * vns[0] + (dps[0] - dps[1])) / (DL + DR);
      if (SL > R(0)) {
#pragma unroll
        for (int v = 0; v < NV; ++v) F[v] = fL[v];
      } else if (!(Ss > R(0)) && !(SR > R(0))) {
#pragma unroll
        for (int v = 0; v < NV; ++v) F[v] = fR[v];
      } else {  // the star regions, sampled in riemann_hllc's order
        const int k = Ss > R(0) ? 0 : 1;
        const R SK = k == 0 ? SL : SR, vK = vns[k], r = rs[k];
        const R q = SK * ((Ss - vK) / (SK - Ss));
        const R *f = k == 0 ? fL : fR;
        F[0] = f[0] + q * r;
        F[N] = f[N] + q * (r * SK);
        F[T] = f[T] + q * (r * vts[k]);
        F[3] = f[3] + q * (Hs[k] + r * Ss * (SK - vK));
      }
    }
  }
}

// FP32 LLF face point on packed pairs (sm_100+ f32x2 arithmetic: one instruction for two
// lanes): d2[v] = (left, right) perturbation traces, the two sides' exact-difference
// fluxes and sound speeds computed side by side.  Returns F[v] = 2 (F_hat - F(u_eq))
// = (f_L + lam d_L) + (f_R - lam d_R); the caller folds the 0.5 into its edge weights.
template <int DIR>
__device__ __forceinline__ void face_point_pk(const StageArgs<float> &A, const float2 *d2,
                                              float re, float pe, float *F) {
  float2 r2 = __fadd2_rn(make_float2(re, re), d2[0]);
  r2.x = rfmax(r2.x, 1.0e-9f);
  r2.y = rfmax(r2.y, 1.0e-9f);
  const float2 inv = make_float2(frcp(r2.x), frcp(r2.y));
  const float2 vx = __fmul2_rn(d2[1], inv), vy = __fmul2_rn(d2[2], inv);
  const float2 ke = __ffma2_rn(d2[2], vy, __fmul2_rn(d2[1], vx));
  const float2 dp = __fmul2_rn(make_float2(A.gm1, A.gm1),
                               __ffma2_rn(make_float2(-0.5f, -0.5f), ke, d2[3]));
  const float hp = A.hgam * pe;
  const float2 H = __fadd2_rn(__fadd2_rn(make_float2(hp, hp), d2[3]), dp);
  const float2 vn = DIR == 0 ? vx : vy;
  float2 f[NV];
  f[0] = d2[1 + DIR];
  f[1] = DIR == 0 ? __ffma2_rn(d2[1], vx, dp) : __fmul2_rn(d2[1], vy);
  f[2] = DIR == 0 ? __fmul2_rn(d2[2], vx) : __ffma2_rn(d2[2], vy, dp);
  f[3] = __fmul2_rn(vn, H);
  float2 pp = __fadd2_rn(make_float2(pe, pe), dp);
  pp.x = rfmax(pp.x, 1e-10f);
  pp.y = rfmax(pp.y, 1e-10f);
  const float2 c2 = __fmul2_rn(__fmul2_rn(make_float2(A.gamma, A.gamma), pp), inv);
  const float cL = fsqrt_pos(c2.x), cR = fsqrt_pos(c2.y);
  float lam;
  if (A.llf_speed == 1)
    lam = rfmax(fabsf(vn.y + cR), fabsf(vn.x + cL));
  else
    lam = rfmax(fabsf(vn.x) + cL, fabsf(vn.y) + cR);
  const float2 l2 = make_float2(lam, -lam);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const float2 g = __ffma2_rn(l2, d2[v], f[v]);
    F[v] = g.x + g.y;
  }
}

// Limit one cell's modes in place (base[m*mstride] is mode m of one variable).
template <typename R, int K, int BASIS>
__device__ __forceinline__ void limit_modes(const StageArgs<R> &A, const StageArgs<R> &I,
                                            R *base, int mstride, R m0,
                                            R mw, R me, R ms, R mn) {
  if constexpr (K >= 1) {
    constexpr int NB = num_modes(K, BASIS);
    constexpr int M10 = mode_index(K, BASIS, 1, 0), M01 = mode_index(K, BASIS, 0, 1);
    R sx = base[M10 * mstride], sy = base[M01 * mstride];
    // minmod of the scaled slope and the mean differences, scaled back by 1 / norm (a
    // product: a division per slope would cost a dozen instructions at every staged cell)
    R l1 = gminmod(A.lim_norm * sx, me - m0, m0 - mw, I.lim_Mdx2) * A.lim_inorm;
    R l2 = gminmod(A.lim_norm * sy, mn - m0, m0 - ms, I.lim_Mdy2) * A.lim_inorm;
    if (fabs(l1 - sx) > A.lim_tol || fabs(l2 - sy) > A.lim_tol) {
      base[M10 * mstride] = l1;
      base[M01 * mstride] = l2;
#pragma unroll
      for (int m = 0; m < NB; ++m)
        if (mode_deg(K, BASIS, m, 0) + mode_deg(K, BASIS, m, 1) >= 2) base[m * mstride] = R(0);
    }
  }
}

// Zhang-Shu positivity limiter on one cell, compute_positivity (2d/limiters.f90:478-654),
// in delta form: the limiter acts on the full-state polynomial W = e + d, e the cell's
// projected equilibrium (density and energy modes; zero momentum), and writes back
// d' = s W - e = s d + (s - 1) e for the non-mean modes, s = theta t for the density and
// t for the other variables.  The positivity set is compute_set's (2d/limiters.f90:438-475):
// Gauss-Lobatto nodes in one direction times Gauss nodes in the other, both ways.
// d[v*NB + m] holds the cell's modes (updated in place); fx / fy are the cell's NQ
// equilibrium factors at the volume points.  A cell the limiter leaves alone
// (theta = t = 1) is not written.  Not inlined: it is off the default path, and its
// point loops stay rolled to keep the stage kernels small.
template <typename R, int K, int BASIS>
__device__ __noinline__ void positivity_cell(const StageArgs<R> &A, const int kind, R *d,
                                             const R *fx, const R *fy) {
  if constexpr (K >= 1) {
    constexpr int NB = num_modes(K, BASIS), NQ = K + 1;
    using T = TC<R, K>;
    constexpr int NG = T::NG;
    R er[NB], ee[NB];
#pragma unroll
    for (int m = 0; m < NB; ++m) er[m] = ee[m] = R(0);
#pragma unroll 1
    for (int qa = 0; qa < NQ; ++qa)
#pragma unroll 1
      for (int qb = 0; qb < NQ; ++qb) {
        R re, pe;
        eq_point(A, kind, fx[qa], fy[qb], re, pe);
        pe *= A.igm1;
        const R w = R(0.25) * T::wq(qa) * T::wq(qb);
#pragma unroll
        for (int m = 0; m < NB; ++m) {
          const int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
          const R bw = w * (T::B(a, qa) * T::B(b, qb));
          er[m] += re * bw;
          ee[m] += pe * bw;
        }
      }
    R W[NV][NB];
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        const R x = d[v * NB + m];
        W[v][m] = v == 0 ? er[m] + x : (v == 3 ? ee[m] + x : x);
      }
    const R eps = A.pos_eps;
    // density: theta = min(|(rho_avg - eps) / (rho_avg - rho_min)|, 1)
    const R rbar = W[0][0];
    R rmin = rbar;
#pragma unroll 1
    for (int p = 0; p < 2 * NQ * NG; ++p) {
      const int fam = p / (NQ * NG), q = (p / NG) % NQ, g = p % NG;
      R r = R(0);
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        const int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
        r += W[0][m] * (fam == 0 ? T::Gl(a, g) * T::B(b, q) : T::B(a, q) * T::Gl(b, g));
      }
      rmin = fmin(rmin, r);
    }
    const R theta = fmin(fabs((rbar - eps) / (rbar - rmin)), R(1));
    // pressure on the density-limited set; solve_for_t (2d/limiters.f90:312-362) where
    // p <= eps
    R tmin = R(1);
#pragma unroll 1
    for (int p = 0; p < 2 * NQ * NG; ++p) {
      const int fam = p / (NQ * NG), q = (p / NG) % NQ, g = p % NG;
      R u[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        R sacc = R(0);
#pragma unroll
        for (int m = 1; m < NB; ++m) {
          const int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
          sacc += W[v][m] * (fam == 0 ? T::Gl(a, g) * T::B(b, q) : T::B(a, q) * T::Gl(b, g));
        }
        u[v] = W[v][0] + (v == 0 ? theta * sacc : sacc);
      }
      const R rf = rfmax(u[0], R(1.0e-9f));
      const R pr = A.gm1 * (u[3] - R(0.5) * (u[1] * u[1] + u[2] * u[2]) / rf);
      if (!(pr > eps)) {
        const R dr = u[0] - W[0][0], dmx = u[1] - W[1][0], dmy = u[2] - W[2][0];
        const R de = u[3] - W[3][0];
        const R qa = R(2) * dr * de - dmx * dmx - dmy * dmy;
        R qb = R(2) * dr * (W[3][0] - eps * A.igm1) + R(2) * W[0][0] * de -
               R(2) * (W[1][0] * dmx + W[2][0] * dmy);
        R qc = R(2) * W[0][0] * W[3][0] - (W[1][0] * W[1][0] + W[2][0] * W[2][0]) -
               R(2) * eps * W[0][0] * A.igm1;
        qb = qb / qa;
        qc = qc / qa;
        const R D = sqrt(fabs(qb * qb - R(4) * qc));
        const R t1 = R(0.5) * (-qb - D), t2 = R(0.5) * (-qb + D);
        R t;
        if (t1 > -eps && t1 < R(1) + eps) t = t1;
        else if (t2 > -eps && t2 < R(1) + eps) t = t2;
        else t = R(0);
        t = fmax(R(0), fmin(R(1), t));
        if (tmin >= t) tmin = t;
      }
    }
    if (theta < R(1) || tmin < R(1)) {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const R sc = v == 0 ? theta * tmin : tmin;
#pragma unroll
        for (int m = 1; m < NB; ++m) {
          const R e = v == 0 ? er[m] : (v == 3 ? ee[m] : R(0));
          d[v * NB + m] = sc * d[v * NB + m] + (sc - R(1)) * e;
        }
      }
    }
  }
}

__device__ __forceinline__ double block_max(double v, double *red, int tid, int nthr) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
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

// ---------------------------------------------------------------- tile staging

template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  // 16-byte chunks bypass L1 (.cg): staged data is read once from shared memory, and
  // allocating it in L1 cost about 13 % of the stage time; 4- and 8-byte copies need .ca
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ---------------------------------------------------------------- TMA tile copies
// One bulk tensor copy stages the modes of an interior tile (tile + one-cell halo, the
// 16-byte aligned x range [i0-4, i0+TX+4)) into the buffer layout [plane][RY][PX]; its
// completion is counted on an mbarrier (expect_tx bytes).  Waits are bounded.
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of `bar`: false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity,
                                          int limit = 1 << 22) {
  for (int it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int x, int y, int z,
                                            unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3, %4}], [%5];\n" ::"r"(smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
// Interior tiles whose staged block lies inside the grid: x range [i0-4, i0+TX+4) (a
// 16-byte aligned start, as TMA requires), rows [j0-1, j0+TY] (no boundary mapping).
template <int TX, int TY>
__device__ __forceinline__ bool tma_tile(const int use_tma, const int nx, const int ny,
                                         const int i0, const int j0) {
  return use_tma && i0 >= 4 && i0 + TX + 4 <= nx && j0 >= 1 && j0 + TY + 1 <= ny;
}

// Issue the asynchronous copies that stage one tile (lower-left cell (i0, j0)) into `buf`:
// the modes of the tile and a one-cell halo, the means of a two-cell halo when the
// limiter is on, and the tile's equilibrium factors.  Boundary conditions are applied by
// index mapping.  The modes are staged by (row, chunk) slots: a thread keeps its slot and
// walks the planes, so the slot's index arithmetic and boundary mapping are done once.
template <typename R, int K, int BASIS, int TX, int TY, int NT = TX * TY>
__device__ __forceinline__ void tile_load_async(const StageArgs<R> &A, const bool lim,
                                                const int i0, const int j0, R *buf,
                                                const int tid, const bool modes = true) {
  constexpr int nthr = NT;  // threads of the CTA
  const TileLayout L = tile_layout(K, BASIS, TX, TY, lim);
  const int nx = A.nx, ny = A.ny, pitch = A.pitch;
  const long long P = A.plane;
  constexpr int PX = TX + 8, RY = TY + 2, RXY = PX * RY;
  constexpr int NPL = NV * num_modes(K, BASIS);  // planes (variable x mode)
  constexpr int VEC = 16 / (int)sizeof(R);       // elements per 16-byte chunk
  constexpr int CPR = PX / VEC;                  // chunks per stored row
  // Slot (ry, ch): stored row ry (grid row j0 + ry - 1, BC-mapped), chunk ch (grid columns
  // c0 = i0 - 4 + ch * VEC .. c0 + VEC - 1) of every plane.  With at least as many threads
  // as slots, PSTEP threads share a slot and take every PSTEP-th plane.
  constexpr int NSLOT = RY * CPR;
  constexpr bool WIDE = nthr >= NSLOT;
  constexpr int PSTEP = WIDE ? nthr / NSLOT : 1;
  // a chunk inside the grid is one 16-byte copy per plane (two 8-byte copies when FP32
  // rows are only 8-byte aligned); a chunk reaching outside stages only the columns the
  // tile reads, [i0 - xr, i0 + TX + xr) (the one-cell ring, two cells deep in x with the
  // limiter), element by element with x mapping
  const bool v16 = (pitch % VEC) == 0 && (P % VEC) == 0;
  const bool v8 = !v16 && VEC == 4 && (pitch % 2) == 0 && (P % 2) == 0;
  const int xr = L.lim ? 2 : 1;
  if (modes) {
    const int ps = WIDE ? tid / NSLOT : 0;  // the slot's first plane
    for (int slot = WIDE ? (tid < PSTEP * NSLOT ? tid % NSLOT : NSLOT) : tid; slot < NSLOT;
         slot += WIDE ? NSLOT : nthr) {
      const int ry = slot / CPR, ch = slot - ry * CPR;
      const int gj = wrap_index(j0 + ry - 1, ny, A.bc_y);
      const int c0 = i0 - 4 + ch * VEC;
      const R *src = A.x + (long long)ps * P + (long long)gj * pitch;
      R *dst = buf + L.su + ps * RXY + ry * PX + ch * VEC;
      const long long sstep = PSTEP * P;
      if (c0 >= 0 && c0 + VEC <= nx && (v16 || v8)) {
        src += c0;
        if (v16) {
#pragma unroll 4
          for (int pl = ps; pl < NPL; pl += PSTEP, src += sstep, dst += PSTEP * RXY)
            cp_async<16>(dst, src);
        } else {
#pragma unroll 4
          for (int pl = ps; pl < NPL; pl += PSTEP, src += sstep, dst += PSTEP * RXY) {
            cp_async<8>(dst, src);
            cp_async<8>(dst + 2, src + 2);
          }
        }
      } else {
        const int lo = max(c0, i0 - xr), hi = min(c0 + VEC, i0 + TX + xr);
        if (lo < hi) {
          int gi[VEC];
#pragma unroll
          for (int e = 0; e < VEC; ++e) gi[e] = lo + e < hi ? wrap_index(lo + e, nx, A.bc_x) : 0;
          dst += lo - c0;
          for (int pl = ps; pl < NPL; pl += PSTEP, src += sstep, dst += PSTEP * RXY) {
#pragma unroll
            for (int e = 0; e < VEC; ++e)
              if (lo + e < hi) cp_async<sizeof(R)>(dst + e, src + gi[e]);
          }
        }
      }
    }
  }
  if (L.lim) {
    // means of the second ring's rows j0 - 2 and j0 + TY + 1 (ring-1 columns)
    constexpr int RXL = TX + 2;
    for (int k = tid; k < NV * 2 * RXL; k += nthr) {
      const int c = k % RXL, t = k / RXL, side = t & 1, v = t >> 1;
      const int gj = wrap_index(side ? j0 + TY + 1 : j0 - 2, ny, A.bc_y);
      const int gi = wrap_index(i0 - 1 + c, nx, A.bc_x);
      cp_async<sizeof(R)>(buf + L.sm + (v * 2 + side) * PX + 3 + c,
                          A.x + (long long)(v * L.NB) * P + (long long)gj * pitch + gi);
    }
  }
  // equilibrium factors: fxv [NQ*(TX+2)] and fyv [NQ*(TY+2)] of the tile and its halo
  // (BC-mapped like the modes), fxf [TX+1] and fyf [TY+1] (indices clamped)
  constexpr int NQ = K + 1;
  constexpr int n1 = NQ * (TX + 2), n2 = n1 + TX + 1, n3 = n2 + NQ * (TY + 2), n4 = n3 + TY + 1;
  R *e = buf + L.eq;
  for (int k = tid; k < n4; k += nthr) {
    const R *src;
    if (k < n1) {
      const int c = k / NQ, q = k - c * NQ;
      src = A.fxv + wrap_index(i0 - 1 + c, nx, A.bc_x) * NQ + q;
    } else if (k < n2) {
      src = A.fxf + min(i0 + (k - n1), nx);
    } else if (k < n3) {
      const int r = (k - n2) / NQ, q = (k - n2) - r * NQ;
      src = A.fyv + wrap_index(j0 - 1 + r, ny, A.bc_y) * NQ + q;
    } else {
      src = A.fyf + min(j0 + (k - n3), ny);
    }
    cp_async<sizeof(R)>(e + k, src);
  }
}

// Compute one staged tile: limiter, face fluxes, cell quadrature, RK combination and the
// wave-speed reduction.  The CTA has TX * TY / CPT threads; thread tid owns the CPT cells
// e = tid + c * (TX * TY / CPT), c < CPT, cell e at (e % TX, e / TX), and computes them one
// after the other (the per-cell state is reused, so registers do not grow with CPT).
// With end_sync it ends with a CTA barrier, after which `buf` and the flux area may be
// reused.  The wave speed goes to speed_acc (the caller reduces later), or by warp atomics
// (warp_speed), or by a CTA reduction and one atomic.
// A holds the launch's constants (physics, boundary conditions, limiter, RK stage flags);
// I the instance: its grid, buffers, spacing, equilibrium kind and run state.  A single
// grid passes its arguments as both; the batched form passes the group's constants as A
// (kernel parameters: free operands) and the item's instance as I.
template <typename R, int K, int BASIS, int TX, int TY, int VAR, int CPT = 1>
__device__ __forceinline__ void tile_compute(const StageArgs<R> &A, const StageArgs<R> &I,
                                             const bool lim_,
                                             const int i0, const int j0, R *buf, R *flux,
                                             double *red, const int tid, const double dt,
                                             R *speed_acc = nullptr,
                                             const bool end_sync = true,
                                             const bool warp_speed = false) {
  constexpr int NQ = K + 1;
  constexpr int NB = num_modes(K, BASIS);
  constexpr bool FP64 = std::is_same<R, double>::value;
  constexpr bool POS = (VAR & WB_VAR_POSITIVITY) != 0;  // positivity limiter compiled in
  constexpr bool HLLC = (VAR & WB_VAR_HLLC) != 0;       // HLLC face flux (else LLF)
  constexpr bool PKF = !FP64 && !HLLC;                  // packed FP32 LLF faces
  using T = TC<R, K>;
  const TileLayout L = tile_layout(K, BASIS, TX, TY, lim_);
  // RX below is the stored row pitch (TX + 8); the staged ring starts at column 3 of each
  // stored row
  constexpr int RX = TX + 8, RY = TY + 2, RXY = RX * RY, RXL = TX + 2;
  static_assert((TX * TY) % (32 * CPT) == 0, "whole warps of CPT cells per thread");
  constexpr int nthr = TX * TY / CPT;  // threads of the CTA
  constexpr int NCELL = TX * TY;
  const int nx = I.nx, ny = I.ny, pitch = I.pitch;
  const long long P = I.plane;
  const bool lim = lim_;
  const int eqk = I.eq_kind;
  R *su = buf + L.su + 3;
  const R *sm = buf + L.sm + 3;  // [NV][2][RX]: means of rows j0 - 2 and j0 + TY + 1
  // volume-point factors are indexed from the tile's first column / row (halo at -1)
  const R *sfxv = buf + L.eq + NQ;
  const R *sfxf = buf + L.eq + NQ * (TX + 2);
  const R *sfyv = sfxf + TX + 1 + NQ;
  const R *sfyf = sfxf + TX + 1 + NQ * (TY + 2);
  const bool pos = POS && A.limiter == 2 && A.lim_y && K >= 1;
  R *sfx = flux;
  const int FXS = TY * (TX + 1);
  R *sfy = sfx + NV * NQ * FXS;
  const int FYS = (TY + 1) * TX;

  // 2. limiter on every staged cell (means never change, so cells are independent)
  if (lim) {
    // neighbour means from the mode-0 planes (never written by the limiter) and, for the
    // ring's first and last rows, from the staged second-ring rows; a thread takes a cell
    // and its four variables (the cell's index arithmetic once, not once per variable)
    for (int e = tid; e < RY * RXL; e += nthr) {
      const int rx = e % RXL, ry = e / RXL;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const R *mp = su + (v * NB) * RXY + ry * RX + rx;  // mode 0 of cell (ry, rx)
        const R *sd = sm + v * 2 * RX + rx;
        const R ms = ry > 0 ? mp[-RX] : sd[0];
        const R mn = ry < RY - 1 ? mp[RX] : sd[RX];
        limit_modes<R, K, BASIS>(A, I, su + (v * NB) * RXY + ry * RX + rx, RXY, mp[0], mp[-1],
                                 mp[1], ms, mn);
      }
    }
    __syncthreads();
  } else if (pos) {
    for (int e = tid; e < RY * RXL; e += nthr) {
      const int rx = e % RXL, ry = e / RXL;
      R *base = su + ry * RX + rx;
      R dl[NV * NB];
#pragma unroll
      for (int k = 0; k < NV * NB; ++k) dl[k] = base[k * RXY];
      positivity_cell<R, K, BASIS>(A, eqk, dl, sfxv + (rx - 1) * NQ, sfyv + (ry - 1) * NQ);
#pragma unroll
      for (int k = 0; k < NV * NB; ++k) base[k * RXY] = dl[k];
    }
    __syncthreads();
  }

  // 3. faces, x and y in one balanced loop: x face (fi, fj) sits between tile cells
  //    fi-1 and fi of row fj; y face (fi, fj) between rows fj-1 and fj of column fi
  // The y faces start at a warp boundary (x range padded to a multiple of 32), so no
  // warp runs both face kinds in one pass: a warp's passes are all x or all y.
  const int FXP = (FXS + 31) & ~31;
  for (int fa = tid; fa < FXP + FYS; fa += nthr) {
    if (fa < FXP) {
    if (fa >= FXS) continue;
    const int f = fa;
    int fi = f % (TX + 1), fj = f / (TX + 1);
    int gfi = i0 + fi, gj = j0 + fj;
    if (gfi > nx || gj >= ny) continue;
    (void)gj;
    if constexpr (PKF) {
      // packed (left, right) pairs through traces, point values and the flux
      float2 clr[NV][NQ];
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
          for (int a = 0; a < NQ; ++a) {
            int m = mode_index(K, BASIS, a, b);
            if (m < 0) continue;
            const R *pm = su + (v * NB + m) * RXY + (fj + 1) * RX;
            s2 = __ffma2_rn(make_float2(pm[fi], pm[fi + 1]), make_float2(T::Ep(a), T::Em(a)), s2);
          }
          clr[v][b] = s2;
        }
      const float fxf = sfxf[fi];
      float2 mom[2][NQ];  // edge moments of the variable pairs (0, 1) and (2, 3)
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        float2 d2[NV];
        float F[NV], re, pe;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
          for (int b = 0; b < NQ; ++b)
            s2 = __ffma2_rn(clr[v][b], make_float2(T::B(b, q), T::B(b, q)), s2);
          d2[v] = s2;
        }
        eq_point(A, eqk, fxf, sfyv[fj * NQ + q], re, pe);
        face_point_pk<0>(A, d2, re, pe, F);
        const float2 Fp[2] = {make_float2(F[0], F[1]), make_float2(F[2], F[3])};
#pragma unroll
        for (int pp = 0; pp < 2; ++pp)
#pragma unroll
          for (int c = 0; c < NQ; ++c) {
            const float w = 0.5f * T::BW(c, q);
            mom[pp][c] = __ffma2_rn(Fp[pp], make_float2(w, w), q == 0 ? make_float2(0.f, 0.f) : mom[pp][c]);
          }
      }
      const float2 h2 = make_float2(I.hidx, I.hidx);
#pragma unroll
      for (int pp = 0; pp < 2; ++pp)
#pragma unroll
        for (int c = 0; c < NQ; ++c) {
          const float2 r2 = __fmul2_rn(mom[pp][c], h2);
          sfx[((2 * pp) * NQ + c) * FXS + f] = r2.x;
          sfx[((2 * pp + 1) * NQ + c) * FXS + f] = r2.y;
        }
    } else {  // FP64, and the FP32 HLLC variant
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
          sl += pm[fi] * T::Ep(a);
          sr += pm[fi + 1] * T::Em(a);
        }
        cl[v][b] = sl;
        cr[v][b] = sr;
      }
    const R fxf = sfxf[fi];
    R mom[NV][NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      R dL[NV], dR[NV], F[NV], re, pe;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        R sl = R(0), sr = R(0);
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          sl += cl[v][b] * T::B(b, q);
          sr += cr[v][b] * T::B(b, q);
        }
        dL[v] = sl;
        dR[v] = sr;
      }
      eq_point(A, eqk, fxf, sfyv[fj * NQ + q], re, pe);
      face_point<R, 0, HLLC>(A, dL, dR, re, pe, F);
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int b = 0; b < NQ; ++b) mom[v][b] = (q == 0 ? R(0) : mom[v][b]) + F[v] * T::BW(b, q);
    }
    // edge moments sum_q F(q) phi_b(eta_q) w_q, scaled by 0.5/dx, shared by both cells
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int b = 0; b < NQ; ++b) sfx[(v * NQ + b) * FXS + f] = mom[v][b] * I.hidx;
    }
    } else {
    const int f = fa - FXP;
    int fi = f % TX, fj = f / TX;
    int gi = i0 + fi, gfj = j0 + fj;
    if (gi >= nx || gfj > ny) continue;
    if constexpr (PKF) {
      // packed (bottom, top) pairs
      float2 cbt[NV][NQ];
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int a = 0; a < NQ; ++a) {
          float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
          for (int b = 0; b < NQ; ++b) {
            int m = mode_index(K, BASIS, a, b);
            if (m < 0) continue;
            const R *pm = su + (v * NB + m) * RXY + (fi + 1);
            s2 = __ffma2_rn(make_float2(pm[fj * RX], pm[(fj + 1) * RX]),
                            make_float2(T::Ep(b), T::Em(b)), s2);
          }
          cbt[v][a] = s2;
        }
      const float fyf = sfyf[fj];
      float2 mom[2][NQ];  // edge moments of the variable pairs (0, 1) and (2, 3)
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        float2 d2[NV];
        float F[NV], re, pe;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
          for (int a = 0; a < NQ; ++a)
            s2 = __ffma2_rn(cbt[v][a], make_float2(T::B(a, q), T::B(a, q)), s2);
          d2[v] = s2;
        }
        eq_point(A, eqk, sfxv[fi * NQ + q], fyf, re, pe);
        face_point_pk<1>(A, d2, re, pe, F);
        const float2 Fp[2] = {make_float2(F[0], F[1]), make_float2(F[2], F[3])};
#pragma unroll
        for (int pp = 0; pp < 2; ++pp)
#pragma unroll
          for (int c = 0; c < NQ; ++c) {
            const float w = 0.5f * T::BW(c, q);
            mom[pp][c] = __ffma2_rn(Fp[pp], make_float2(w, w), q == 0 ? make_float2(0.f, 0.f) : mom[pp][c]);
          }
      }
      const float2 h2 = make_float2(I.hidy, I.hidy);
#pragma unroll
      for (int pp = 0; pp < 2; ++pp)
#pragma unroll
        for (int c = 0; c < NQ; ++c) {
          const float2 r2 = __fmul2_rn(mom[pp][c], h2);
          sfy[((2 * pp) * NQ + c) * FYS + f] = r2.x;
          sfy[((2 * pp + 1) * NQ + c) * FYS + f] = r2.y;
        }
    } else {  // FP64, and the FP32 HLLC variant
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
          sb += pm[fj * RX] * T::Ep(b);
          st += pm[(fj + 1) * RX] * T::Em(b);
        }
        cb[v][a] = sb;
        ct[v][a] = st;
      }
    const R fyf = sfyf[fj];
    R mom[NV][NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      R dB[NV], dT[NV], F[NV], re, pe;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        R sb = R(0), st = R(0);
#pragma unroll
        for (int a = 0; a < NQ; ++a) {
          sb += cb[v][a] * T::B(a, q);
          st += ct[v][a] * T::B(a, q);
        }
        dB[v] = sb;
        dT[v] = st;
      }
      eq_point(A, eqk, sfxv[fi * NQ + q], fyf, re, pe);
      face_point<R, 1, HLLC>(A, dB, dT, re, pe, F);
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int a = 0; a < NQ; ++a) mom[v][a] = (q == 0 ? R(0) : mom[v][a]) + F[v] * T::BW(a, q);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int a = 0; a < NQ; ++a) sfy[(v * NQ + a) * FYS + f] = mom[v][a] * I.hidy;
    }
    }
  }
  __syncthreads();

  // 4. cells
  // wave-speed maxima in the kernel's precision (a maximum of floats is exact; FP64
  // arithmetic is slow on this part), widened to double only for the atomics
  R spx = R(0), spy = R(0);
#pragma unroll 1
  for (int cc = 0; cc < CPT; ++cc) {
  const int ce = tid + cc * nthr;  // the thread's cc-th cell of the tile
  const int tx = ce % TX, ty = ce / TX;
  const int gi = i0 + tx, gj = j0 + ty;
  const bool active = gi < nx && gj < ny;
  const R *uc = su + (ty + 1) * RX + (tx + 1);  // mode m of var v at uc[(v*NB+m)*RXY]
  R acc[NV][NB];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int m = 0; m < NB; ++m) acc[v][m] = R(0);
  R rbar = R(0), pbar = R(0);
  // The first RK input of the first output (U^n of SSP-RK2's second stage) is staged into
  // the face-flux area once the edge integrals have read it, so its loads land during the
  // volume quadrature instead of stalling the RK combination.  FP32, where the tile's
  // modes fit the flux area (not the tensor P2 basis).
  // (One cell per thread only: with several, the face fluxes are still being read by the
  // thread's later cells.)
  constexpr bool UN = CPT == 1 && !FP64 &&
                      NV * NB * TX * TY <= NV * NQ * (TY * (TX + 1) + (TY + 1) * TX);
  const bool un = UN && I.o[0].out != nullptr && I.o[0].in[0] != nullptr;
  R *sun = flux;  // [NV*NB][TX*TY]
  // With the minmod limiter on that input (SSP-RK2's U^n), the means of its one-cell ring
  // are staged behind it, [NV][W: TY, E: TY, S: TX, N: TX], so the limiter of U^n reads
  // every neighbour mean from shared memory (full tiles; a tile cut by the grid's edge
  // reads them from global memory).
  constexpr int RING = 2 * (TX + TY);
  constexpr bool UNL = UN && K >= 1 &&
                       NV * NB * TX * TY + NV * RING <= NV * NQ * (TY * (TX + 1) + (TY + 1) * TX);
  const bool full = i0 + TX <= nx && j0 + TY <= ny;
  const bool unl = UNL && un && full && I.o[0].lim[0] && A.limiter == 1;
  R *sring = sun + NV * NB * NCELL;
  auto source_edges = [&]() {
    if constexpr (!FP64) {
      // FP32 form: the gravity source (0, -gx drho, -gy drho, -(gx m_x + gy m_y)) is linear
      // in the perturbation, so its Gauss projection is exactly -g times the modes
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        const R r = uc[(0 * NB + m) * RXY], mx = uc[(1 * NB + m) * RXY];
        const R my = uc[(2 * NB + m) * RXY];
        acc[1][m] -= A.gx * r;
        acc[2][m] -= A.gy * r;
        acc[3][m] -= A.gx * mx + A.gy * my;
      }
    }
    // edge integrals: the faces' moments (already weighted by 0.5/dx, 0.5/dy)
    const int fl = ty * (TX + 1) + tx, fb = ty * TX + tx;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      R FR[NQ], FL[NQ], GT[NQ], GB[NQ];
#pragma unroll
      for (int b = 0; b < NQ; ++b) {
        FR[b] = sfx[(v * NQ + b) * FXS + fl + 1];
        FL[b] = sfx[(v * NQ + b) * FXS + fl];
        GT[b] = sfy[(v * NQ + b) * FYS + fb + TX];
        GB[b] = sfy[(v * NQ + b) * FYS + fb];
      }
      // phi_a(-1) = (-1)^a phi_a(+1): the x term of mode (a, b) is phi_a(1) (FR - FL) for
      // even a and phi_a(1) (FR + FL) for odd a, so the sums and differences are formed once
      // per (parity, b) and shared by the modes
      R XD[NQ], XS[NQ], YD[NQ], YS[NQ];
#pragma unroll
      for (int b = 0; b < NQ; ++b) {
        XD[b] = FR[b] - FL[b];
        XS[b] = FR[b] + FL[b];
        YD[b] = GT[b] - GB[b];
        YS[b] = GT[b] + GB[b];
      }
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
        const R ex = (a & 1) ? XS[b] : XD[b], ey = (b & 1) ? YS[a] : YD[a];
        acc[v][m] -= T::Ep(a) * ex + T::Ep(b) * ey;
      }
    }

  };
  if (un) {
    if (active) source_edges();
    __syncthreads();  // every thread is done with the face fluxes
    const R *in0 = I.o[0].in[0];
    if (full && (pitch % 4) == 0) {
      // 16-byte chunks: a thread keeps its (row, chunk) and walks the planes
      constexpr int CPR_U = TX / 4, PCH = TY * CPR_U, NCH = NV * NB * PCH;
      if constexpr (nthr % PCH == 0) {
        const int q = tid % PCH, r = q / CPR_U, ch = q - r * CPR_U;
        const R *src = in0 + (long long)(j0 + r) * pitch + i0 + ch * 4;
        R *dst = sun + r * TX + ch * 4;
        for (int pl = tid / PCH; pl < NV * NB; pl += nthr / PCH)
          cp_async<16>(dst + pl * NCELL, src + pl * P);
      } else {
        for (int k = tid; k < NCH; k += nthr) {
          const int row = k / CPR_U, ch = k - row * CPR_U;
          const int pl = row / TY, r = row - pl * TY;
          cp_async<16>(sun + pl * NCELL + r * TX + ch * 4,
                       in0 + pl * P + (long long)(j0 + r) * pitch + i0 + ch * 4);
        }
      }
    } else if (active) {
      const long long c0 = (long long)gj * pitch + gi;
#pragma unroll
      for (int pl = 0; pl < NV * NB; ++pl) cp_async<sizeof(R)>(sun + pl * NCELL + ce, in0 + pl * P + c0);
    }
    if (unl) {  // the ring's means (boundary conditions by index mapping)
      for (int k = tid; k < NV * RING; k += nthr) {
        const int v = k / RING, e = k - v * RING;
        int gx, gy;
        if (e < 2 * TY) {
          gx = e < TY ? i0 - 1 : i0 + TX;
          gy = j0 + (e < TY ? e : e - TY);
        } else {
          const int f = e - 2 * TY;
          gx = i0 + (f < TX ? f : f - TX);
          gy = f < TX ? j0 - 1 : j0 + TY;
        }
        gx = wrap_index(gx, nx, A.bc_x);
        gy = wrap_index(gy, ny, A.bc_y);
        cp_async<sizeof(R)>(sring + k, in0 + (long long)(v * NB) * P + (long long)gy * pitch + gx);
      }
    }
    cp_async_commit();
  }
  if (active) {
    // The FP64 qa loop stays rolled (a third of the code, fewer instruction-fetch stalls);
    // the packed FP32 loop is short enough to unroll, which measured 1 % faster.
    if constexpr (!FP64) {
      // FP32 on packed pairs: point values as (rho, E) and (m_x, m_y), split fluxes as
      // (Fx, Fy) of one variable, projections as (P_b, Q_{b+1}) with P_b = sum Fx BW(b),
      // Q_b = sum Fy DW(b) (the 0.5/dy goes into bwy below)
#pragma unroll
      for (int qa = 0; qa < NQ; ++qa) {
        float2 cre[NQ], cmm[NQ];
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          float2 s1 = make_float2(0.f, 0.f), s2 = make_float2(0.f, 0.f);
#pragma unroll
          for (int a = 0; a < NQ; ++a) {
            int m = mode_index(K, BASIS, a, b);
            if (m < 0) continue;
            const float2 B2 = make_float2(T::B(a, qa), T::B(a, qa));
            s1 = __ffma2_rn(make_float2(uc[(0 * NB + m) * RXY], uc[(3 * NB + m) * RXY]), B2, s1);
            s2 = __ffma2_rn(make_float2(uc[(1 * NB + m) * RXY], uc[(2 * NB + m) * RXY]), B2, s2);
          }
          cre[b] = s1;
          cmm[b] = s2;
        }
        const float fx = sfxv[tx * NQ + qa];
        float2 PQ[NV][K > 0 ? K : 1];
        float PK[NV];  // P_K, needed by the tensor basis only
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          PK[v] = 0.f;
#pragma unroll
          for (int b = 0; b < K; ++b) PQ[v][b] = make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int qb = 0; qb < NQ; ++qb) {
          float2 dre = make_float2(0.f, 0.f), dm = make_float2(0.f, 0.f);
#pragma unroll
          for (int b = 0; b < NQ; ++b) {
            const float2 B2 = make_float2(T::B(b, qb), T::B(b, qb));
            dre = __ffma2_rn(cre[b], B2, dre);
            dm = __ffma2_rn(cmm[b], B2, dm);
          }
          float re, pe;
          eq_point(A, eqk, fx, sfyv[ty * NQ + qb], re, pe);
          if (A.compute_speed) {
            float ww = 0.25f * T::wq(qa) * T::wq(qb);
            rbar += re * ww;
            pbar += pe * ww;
          }
          // split fluxes by exact differences about a static equilibrium (u_eq velocity 0),
          // x and y side by side:  d(rho u) = m_x,  d(rho u^2 + p) = m_x^2 / rho + dp,
          // d(rho u v) = m_x m_y / rho,  d(u (E + p)) = u (H_eq + dE + dp),
          // dp = (gamma - 1)(dE - |m|^2 / (2 rho))
          const float r = rfmax(re + dre.x, 1.0e-9f);
          const float inv = frcp(r);
          const float2 vel = __fmul2_rn(dm, make_float2(inv, inv));
          const float dp = A.gm1 * (dre.y - 0.5f * (dm.x * vel.x + dm.y * vel.y));
          const float H = A.hgam * pe + dre.y + dp;
          float2 F[NV];
          F[0] = dm;
          F[1] = __ffma2_rn(make_float2(dm.x, dm.x), vel, make_float2(dp, 0.f));
          F[2] = __ffma2_rn(make_float2(dm.y, dm.y), vel, make_float2(0.f, dp));
          F[3] = __fmul2_rn(vel, make_float2(H, H));
#pragma unroll
          for (int b = 0; b < K; ++b) {
            const float2 W2 = make_float2(T::BW(b, qb), T::DW(b + 1, qb));
#pragma unroll
            for (int v = 0; v < NV; ++v) PQ[v][b] = __ffma2_rn(F[v], W2, PQ[v][b]);
          }
          if constexpr (BASIS == 0) {
#pragma unroll
            for (int v = 0; v < NV; ++v) PK[v] += F[v].x * T::BW(K, qb);
          }
        }
        float dwx[NQ], bwy[NQ];
#pragma unroll
        for (int a = 0; a < NQ; ++a) {
          dwx[a] = I.hidx * T::DW(a, qa);
          bwy[a] = I.hidy * T::BW(a, qa);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
          for (int m = 0; m < NB; ++m) {
            constexpr int dummy = 0;
            (void)dummy;
            int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
            if (b > 0) acc[v][m] += bwy[a] * PQ[v][b - 1].y;
            if (a > 0) acc[v][m] += dwx[a] * (b < K ? PQ[v][b].x : PK[v]);
          }
      }
    } else {
#pragma unroll 1
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
            s += uc[(v * NB + m) * RXY] * T::B(a, qa);
          }
          c[v][b] = s;
        }
      const R fx = sfxv[tx * NQ + qa];
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
          for (int b = 0; b < NQ; ++b) s += c[v][b] * T::B(b, qb);
          d[v] = s;
        }
        eq_point(A, eqk, fx, sfyv[ty * NQ + qb], re, pe);
        if (A.compute_speed) {
          R ww = R(0.25) * T::wq(qa) * T::wq(qb);
          rbar += re * ww;
          pbar += pe * ww;
        }
        vol_point(A, d, re, pe, Fx, Fy, S);
        // x fluxes are weighted by 0.5/dx once per qa below; y fluxes take 0.5/dy here
#pragma unroll
        for (int b = 0; b < NQ; ++b) {
          const R dwy = b > 0 ? I.hidy * T::DW(b, qb) : R(0);
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            if (BASIS == 0 || b < K) Pq[v][b] += Fx[v] * T::BW(b, qb);
            if constexpr (FP64) Qq[v][b] += S[v] * T::BW(b, qb);
            if (b > 0) Qq[v][b] += Fy[v] * dwy;
          }
        }
      }
      R dwx[NQ];
#pragma unroll
      for (int a = 0; a < NQ; ++a) dwx[a] = I.hidx * T::DW(a, qa);
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int m = 0; m < NB; ++m) {
          constexpr int dummy = 0;
          (void)dummy;
          int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
          if (FP64 || b > 0) acc[v][m] += T::BW(a, qa) * Qq[v][b];
          if (a > 0) acc[v][m] += dwx[a] * Pq[v][b];
        }
    }
    }
    if (!un) source_edges();
  }
  if (un) {
    cp_async_wait<0>();
    __syncthreads();
  }
  if (active) {
    // RK stage combination: out = sum c_i [lim](in_i) + beta Y + (cdt dt) L(Y).  The RK
    // inputs are read once and the outputs not re-read by this launch: streaming (.cs)
    // loads and stores keep them from displacing the staged halos in L1/L2.
    const long long cell = (long long)gj * pitch + gi;
#pragma unroll
    for (int oi = 0; oi < 2; ++oi) {
      const Combo<R> &o = I.o[oi];
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
        if (un && oi == 0 && ii == 0) {
#pragma unroll
          for (int v = 0; v < NV; ++v)
#pragma unroll
            for (int m = 0; m < NB; ++m) w[v][m] = sun[(v * NB + m) * NCELL + ce];
        } else {
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
          for (int m = 0; m < NB; ++m) w[v][m] = __ldcs(in + (long long)(v * NB + m) * P + cell);
        }
        if (POS && o.lim[ii] && A.limiter == 2 && K >= 1) {
          R dl[NV * NB];
#pragma unroll
          for (int v = 0; v < NV; ++v)
#pragma unroll
            for (int m = 0; m < NB; ++m) dl[v * NB + m] = w[v][m];
          positivity_cell<R, K, BASIS>(A, eqk, dl, sfxv + tx * NQ, sfyv + ty * NQ);
#pragma unroll
          for (int v = 0; v < NV; ++v)
#pragma unroll
            for (int m = 0; m < NB; ++m) w[v][m] = dl[v * NB + m];
        } else if (unl && oi == 0 && ii == 0) {
          // U^n's neighbour means from the staged tile (mode 0) and its staged ring
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const R *m0 = sun + (v * NB) * NCELL + ce;
            const R *rg = sring + v * RING;
            const R mw = tx > 0 ? m0[-1] : rg[ty];
            const R me = tx < TX - 1 ? m0[1] : rg[TY + ty];
            const R ms = ty > 0 ? m0[-TX] : rg[2 * TY + tx];
            const R mn = ty < TY - 1 ? m0[TX] : rg[2 * TY + TX + tx];
            limit_modes<R, K, BASIS>(A, I, &w[v][0], 1, w[v][0], mw, me, ms, mn);
          }
        } else if (o.lim[ii] && A.limiter == 1 && K >= 1) {
          int iw = wrap_index(gi - 1, nx, A.bc_x), ie = wrap_index(gi + 1, nx, A.bc_x);
          int js = wrap_index(gj - 1, ny, A.bc_y), jn = wrap_index(gj + 1, ny, A.bc_y);
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const R *m0p = in + (long long)(v * NB) * P;
            limit_modes<R, K, BASIS>(A, I, &w[v][0], 1, w[v][0], m0p[(long long)gj * pitch + iw],
                                     m0p[(long long)gj * pitch + ie],
                                     m0p[(long long)js * pitch + gi],
                                     m0p[(long long)jn * pitch + gi]);
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
          __stcs(o.out + (long long)(v * NB + m) * P + cell, r);
          if (oi == 0) val[v][m] = r;  // keep o[0]'s means for the wave speed
        }
      if (oi == 0 && A.compute_speed) {
        // wave speed from the new cell mean of the full state
        R r, p, cx, cy;
        mean_wave_speed(A, rbar, pbar, val[0][0], val[1][0], val[2][0], val[3][0], r, p, cx, cy);
        bool bad = !(r > R(0)) || !(p > R(0)) || !isfinite(cx) || !isfinite(cy);
        if (I.eq_kind == 0) bad = !isfinite(cx) || !isfinite(cy);
        if (bad) atomicOr(&I.dev->err, 1);
        if (isfinite(cx)) spx = rfmax(spx, cx);
        if (isfinite(cy)) spy = rfmax(spy, cy);
      }
    }
  }
  }  // cells of this thread
  if (A.compute_speed) {
    if (speed_acc) {  // the caller reduces once after its last tile
      speed_acc[0] = fmax(speed_acc[0], spx);
      speed_acc[1] = fmax(speed_acc[1], spy);
    } else if (warp_speed) {  // one atomic per warp and no CTA barrier (batched form)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        spx = fmax(spx, __shfl_xor_sync(0xffffffffu, spx, o));
        spy = fmax(spy, __shfl_xor_sync(0xffffffffu, spy, o));
      }
      if ((tid & 31) == 0) {
        atomicMax(&I.dev->smax[I.parity ^ 1][0], (unsigned long long)__double_as_longlong((double)spx));
        atomicMax(&I.dev->smax[I.parity ^ 1][1], (unsigned long long)__double_as_longlong((double)spy));
      }
    } else {
      double mx = block_max((double)spx, red, tid, nthr);
      double my = block_max((double)spy, red, tid, nthr);
      if (tid == 0) {
        atomicMax(&I.dev->smax[I.parity ^ 1][0], (unsigned long long)__double_as_longlong(mx));
        atomicMax(&I.dev->smax[I.parity ^ 1][1], (unsigned long long)__double_as_longlong(my));
      }
    }
  }
  if (end_sync) __syncthreads();
}

// Persistent stage kernel: CTAs stride over the tiles of the grid; the next-but-one
// tile is staged by cp.async while the current one is computed (double buffering).
// The tile shape is a compile-time parameter so all shared-memory indexing folds.
// VAR selects compile-time variants (WB_VAR_*): the positivity limiter (limiter 2) and the
// HLLC face flux; the default kernel carries neither.
template <typename R, int K, int BASIS, int TX, int TY, int VAR, int CPT>
__global__ void __launch_bounds__(TX *TY / CPT, std::is_same<R, float>::value ? 2 : 1)
    k_stage(const __grid_constant__ StageArgs<R> A, const __grid_constant__ CUtensorMap tmap) {
  constexpr int NT = TX * TY / CPT;  // threads: CPT cells each
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  const bool lim = A.limiter == 1 && A.lim_y && K >= 1;  // minmod: stage the means halo
  const TileLayout L = tile_layout(K, BASIS, TX, TY, lim);
  double *red = reinterpret_cast<double *>(smem_raw);
  // two mbarriers (one per staging buffer) after the reduction scratch
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw) + 48;
  R *bufs = reinterpret_cast<R *>(smem_raw + 64 * sizeof(double));
  R *flux = bufs + 2 * L.buf;
  const int nx = A.nx, ny = A.ny;
  const int ntx = (nx + TX - 1) / TX, nty = (ny + TY - 1) / TY, ntiles = ntx * nty;
  const unsigned tma_bytes = (unsigned)(NV * L.NB * L.RY * L.PX * sizeof(R));
  const double dt = stage_dt(A);
  if (A.advance_time && blockIdx.x == 0 && tid == 0) {
    DevState *S = A.dev;
    S->t[A.parity ^ 1] = S->t[A.parity] + dt;
    S->nstep[A.parity ^ 1] = S->nstep[A.parity] + (dt > 0.0 ? 1 : 0);
    S->smax[A.parity ^ 1][0] = 0ull;
    S->smax[A.parity ^ 1][1] = 0ull;
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  // stage tile `tl` into buffer b: one TMA copy for an interior tile's modes (thread 0
  // arms the buffer's mbarrier), cp.async for the rest
  // TMA destinations must be 128-byte aligned: checked, never assumed
  const int use_tma = A.use_tma && (smem_u32(bufs) & 127u) == 0u &&
                      ((L.buf * (int)sizeof(R)) & 127) == 0;
  bool pending[2] = {false, false};  // a TMA copy into buffer b not yet waited for
  unsigned phase[2] = {0u, 0u};
  auto stage = [&](const int i0, const int j0, const int b) {
    R *buf = bufs + b * L.buf;
    const bool tma = tma_tile<TX, TY>(use_tma, nx, ny, i0, j0);
    if (tma && tid == 0) {
      mbar_expect_tx(&bar[b], tma_bytes);
      tma_load_3d(buf + L.su, &tmap, i0 - 4, j0 - 1, 0, &bar[b]);
    }
    pending[b] = tma;
    tile_load_async<R, K, BASIS, TX, TY, NT>(A, lim, i0, j0, buf, tid, !tma);
  };
  bool ok = true;
  R speed[2] = {R(0), R(0)};  // this thread's wave-speed maxima over its tiles
  // Pipeline: tile t is staged while tile t - G is computed.  The barrier after tile t's
  // data arrives also frees tile t - G's buffer and the flux area, so the next tile's
  // copies are issued right after it and tile_compute needs no closing barrier.
  const int G = gridDim.x;
  int t = blockIdx.x;
  // Tile t lies in row t / ntx; within a row the columns are taken in an order rotated by
  // the row index, so that a CTA's tiles t, t + G, t + 2G, ... do not keep to one column when
  // G is a multiple of ntx (the boundary columns, staged element by element, would then all
  // fall to the same CTAs).  The CTAs still work on one compact band of rows at a time.
  // The coordinates of t and of t + G are stepped without a division per tile.
  struct Walk {
    int px, cy, cys;  // t % ntx, t / ntx, (t / ntx) % ntx
  };
  const int gq = G / ntx, gr = G - (G / ntx) * ntx, gqm = gq % ntx;
  auto advance = [&](Walk &w) {
    w.px += gr;
    w.cy += gq;
    w.cys += gqm;
    if (w.px >= ntx) {
      w.px -= ntx;
      ++w.cy;
      ++w.cys;
    }
    if (w.cys >= ntx) w.cys -= ntx;
  };
  auto col = [&](const Walk &w) { return w.px + w.cys >= ntx ? w.px + w.cys - ntx : w.px + w.cys; };
  Walk cur{t % ntx, t / ntx, (t / ntx) % ntx};  // tile t
  Walk nxt = cur;                               // tile t + G
  advance(nxt);
  if (t < ntiles) stage(col(cur) * TX, cur.cy * TY, 0);
  cp_async_commit();
  for (int k = 0; t < ntiles; t += G, ++k) {
    const int b = k & 1;
    cp_async_wait<0>();
    if (pending[b]) {
      if (mbar_wait(&bar[b], phase[b])) {
        phase[b] ^= 1u;
        pending[b] = false;
      } else {  // stays pending: the exit path waits for it once more
        atomicOr(&A.dev->err, 2);
        ok = false;
      }
    }
    if (__syncthreads_or(!ok)) break;
    if (t + G < ntiles) stage(col(nxt) * TX, nxt.cy * TY, b ^ 1);
    cp_async_commit();
    R *buf = bufs + b * L.buf;
    tile_compute<R, K, BASIS, TX, TY, VAR, CPT>(A, A, lim, col(cur) * TX, cur.cy * TY, buf,
                                                flux, red, tid, dt, speed, false);
    cur = nxt;
    advance(nxt);
  }
  __syncthreads();  // the last tile's readers are done before the reduction reuses `red`
  // wave-speed maxima of all this CTA's tiles: one block reduction per launch
  if (A.compute_speed) {
    const double mx = block_max((double)speed[0], red, tid, NT);
    const double my = block_max((double)speed[1], red, tid, NT);
    if (tid == 0) {
      atomicMax(&A.dev->smax[A.parity ^ 1][0], (unsigned long long)__double_as_longlong(mx));
      atomicMax(&A.dev->smax[A.parity ^ 1][1], (unsigned long long)__double_as_longlong(my));
    }
  }
  // nothing may still be copying into shared memory when the CTA exits
  for (int b = 0; b < 2; ++b)
    if (pending[b]) (void)mbar_wait(&bar[b], phase[b]);
  cp_async_wait<0>();
}

}  // namespace wb
