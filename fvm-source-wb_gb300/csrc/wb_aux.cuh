// wb_aux.cuh -- per-cell auxiliary kernels: standalone limiter, wave-speed maxima,
// seeded initial perturbation, precision/layout conversion, FP64 norms and sums.
// Included by the per-precision translation units after wb_stage.cuh.
#pragma once
#include "wb_stage.cuh"

namespace wb {


__device__ __forceinline__ void eq_point64(const AuxArgs &A, double fx, double fy, double &re,
                                           double &pe) {
  if (A.eq_kind == 1) {
    double t = fx * fy;
    re = A.rho0 * t;
    pe = A.p0 * t;
  } else if (A.eq_kind == 2) {
    double s = fx + fy;
    re = pow(s, A.npoly);
    pe = A.kpoly * (re * s);
  } else {
    re = 0.0;
    pe = 0.0;
  }
}

// In-place moment limiter (apply_limiter): means are never modified, so each cell
// reads its neighbours' means and rewrites only its own higher modes.
template <typename R, int K, int BASIS>
__global__ void k_limit(const __grid_constant__ StageArgs<R> A, R *u) {
  constexpr int NB = num_modes(K, BASIS);
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  if (gi >= A.nx || gj >= A.ny || K < 1) return;
  const long long P = A.plane, nx = A.pitch;  // row stride
  const long long cell = gj * nx + gi;
  if (A.limiter == 2) {
    constexpr int NQ = K + 1;
    R fx[NQ], fy[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      fx[q] = A.fxv[gi * NQ + q];
      fy[q] = A.fyv[gj * NQ + q];
    }
    R dl[NV * NB];
#pragma unroll
    for (int k = 0; k < NV * NB; ++k) dl[k] = u[(long long)k * P + cell];
    positivity_cell<R, K, BASIS>(A, A.eq_kind, dl, fx, fy);
#pragma unroll
    for (int k = 1; k < NV * NB; ++k)
      if (k % NB) u[(long long)k * P + cell] = dl[k];
    return;
  }
  int iw = wrap_index(gi - 1, A.nx, A.bc_x), ie = wrap_index(gi + 1, A.nx, A.bc_x);
  int js = wrap_index(gj - 1, A.ny, A.bc_y), jn = wrap_index(gj + 1, A.ny, A.bc_y);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    R w[NB];
#pragma unroll
    for (int m = 0; m < NB; ++m) w[m] = u[(long long)(v * NB + m) * P + cell];
    const R *m0 = u + (long long)(v * NB) * P;
    limit_modes<R, K, BASIS>(A, A, w, 1, w[0], m0[gj * nx + iw], m0[gj * nx + ie], m0[js * nx + gi],
                             m0[jn * nx + gi]);
#pragma unroll
    for (int m = 1; m < NB; ++m) u[(long long)(v * NB + m) * P + cell] = w[m];
  }
}

// Wave-speed maxima of the cell means (compute_max_speed) into dev->smax[parity].
template <typename R, int K, int BASIS>
__global__ void k_max_speed(const __grid_constant__ StageArgs<R> A, const R *u) {
  constexpr int NB = num_modes(K, BASIS), NQ = K + 1;
  __shared__ double red[64];
  const Tab1D<R> &T = c_tab[K];
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  double spx = 0.0, spy = 0.0;
  if (gi < A.nx && gj < A.ny) {
    const long long cell = (long long)gj * A.pitch + gi;
    R rbar = R(0), pbar = R(0);
#pragma unroll
    for (int qa = 0; qa < NQ; ++qa)
#pragma unroll
      for (int qb = 0; qb < NQ; ++qb) {
        R re, pe;
        eq_point(A, A.fxv[gi * NQ + qa], A.fyv[gj * NQ + qb], re, pe);
        R ww = R(0.25) * T.wq[qa] * T.wq[qb];
        rbar += re * ww;
        pbar += pe * ww;
      }
    R d0 = u[(long long)(0 * NB) * A.plane + cell], d1 = u[(long long)(1 * NB) * A.plane + cell];
    R d2 = u[(long long)(2 * NB) * A.plane + cell], d3 = u[(long long)(3 * NB) * A.plane + cell];
    R r, p, sx, sy;
    mean_wave_speed(A, rbar, pbar, d0, d1, d2, d3, r, p, sx, sy);
    spx = (double)sx;
    spy = (double)sy;
    if (!isfinite(spx) || !isfinite(spy)) {
      atomicOr(&A.dev->err, 1);
      spx = spy = 0.0;
    }
  }
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  double mx = block_max(spx, red, tid, nthr), my = block_max(spy, red, tid, nthr);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    atomicMax(&A.dev->smax[A.parity][0], (unsigned long long)__double_as_longlong(mx));
    atomicMax(&A.dev->smax[A.parity][1], (unsigned long long)__double_as_longlong(my));
  }
}

// Seeded perturbation projected onto the modes in FP64, stored in R.
// The pressure bump follows the 'eta' term of 2d/benchmark_2d_dg.f90:145-153; the
// velocity field adds kinetic energy at unchanged rho and p (compute_conservative).
template <typename R, int K, int BASIS>
__global__ void k_init_ic(const __grid_constant__ AuxArgs A, const __grid_constant__ IcArgs I,
                          const Tab1D<double> *Td, R *u) {
  constexpr int NB = num_modes(K, BASIS), NQ = K + 1;
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  if (gi >= A.nx || gj >= A.ny) return;
  const Tab1D<double> &T = Td[K];
  double acc[NV][NB];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int m = 0; m < NB; ++m) acc[v][m] = 0.0;
  const double tpi = 6.283185307179586476925286766559;
  for (int qa = 0; qa < NQ; ++qa)
    for (int qb = 0; qb < NQ; ++qb) {
      double x = ((double)gi + 0.5) * A.dx + A.dx / 2.0 * T.xq[qa];
      double y = ((double)gj + 0.5) * A.dy + A.dy / 2.0 * T.xq[qb];
      double re, pe;
      eq_point64(A, A.fxv[gi * NQ + qa], A.fyv[gj * NQ + qb], re, pe);
      double d[NV] = {0.0, 0.0, 0.0, 0.0};
      if (I.kind == 1) {
        double rx = x - I.xc, ry = y - I.yc;
        double dp = I.amp * exp(-(rx * rx + ry * ry) / (2.0 * I.sigma * I.sigma));
        d[3] = dp * (1.0 / (A.gamma - 1.0));
      } else if (I.kind == 2) {
        double du = 0.0, dv = 0.0;
        for (int m = 0; m < I.nmodes; ++m) {
          double arg = tpi * (I.kx[m] * x + I.ky[m] * y);
          du += I.wt[m] * sin(arg + I.pu[m]);
          dv += I.wt[m] * sin(arg + I.pv[m]);
        }
        du *= I.amp;
        dv *= I.amp;
        d[1] = re * du;
        d[2] = re * dv;
        d[3] = 0.5 * re * (du * du + dv * dv);
      }
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        int a = mode_deg(K, BASIS, m, 0), b = mode_deg(K, BASIS, m, 1);
        double w = T.B[a][qa] * T.B[b][qb] * T.wq[qa] * T.wq[qb];
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v][m] += 0.25 * d[v] * w;
      }
    }
  const long long cell = (long long)gj * A.pitch + gi;
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int m = 0; m < NB; ++m) u[(long long)(v * NB + m) * A.plane + cell] = (R)acc[v][m];
}

// Element-wise precision conversion over nplanes padded planes.
template <typename Ro, typename Ri>
__global__ void k_convert(Ro *out, const Ri *in, long long n) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (; e < n; e += stride) out[e] = (Ro)in[e];
}

// SoA (padded planes) <-> Fortran u(nvar, nx, ny, k+1, k+1) column-major (tensor basis).
template <typename R, int K>
__global__ void k_soa_to_fortran(const R *soa, double *f, int nx, int ny, long long P) {
  constexpr int NQ = K + 1, NB = NQ * NQ;
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  if (gi >= nx || gj >= ny) return;
  const long long cell = (long long)gj * nx + gi;
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    int a = mode_deg(K, 0, m, 0), b = mode_deg(K, 0, m, 1);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      f[v + NV * ((long long)gi + (long long)nx * (gj + (long long)ny * (a + NQ * b)))] =
          (double)soa[(long long)(v * NB + m) * P + cell];
  }
}
template <typename R, int K>
__global__ void k_fortran_to_soa(const double *f, R *soa, int nx, int ny, long long P) {
  constexpr int NQ = K + 1, NB = NQ * NQ;
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  if (gi >= nx || gj >= ny) return;
  const long long cell = (long long)gj * nx + gi;
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    int a = mode_deg(K, 0, m, 0), b = mode_deg(K, 0, m, 1);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      soa[(long long)(v * NB + m) * P + cell] =
          (R)f[v + NV * ((long long)gi + (long long)nx * (gj + (long long)ny * (a + NQ * b)))];
  }
}

}  // namespace wb

namespace wb {

// FP64 error norms of a - b (b may be null) at the GL nodes, compute_error
// (2d/benchmark_2d_dg.f90:23-89): per block partial sums [block][v][0..2] =
// (L1 sum, L2 sum, Linf), reduced in a fixed order by k_norms_final.
template <int K, int BASIS>
__global__ void k_norms(const __grid_constant__ AuxArgs A, const Tab1D<double> *Td, const double *a,
                        const double *b, double *partial) {
  constexpr int NB = num_modes(K, BASIS), NQ = K + 1;
  __shared__ double red[NV * 3][64];
  const Tab1D<double> &T = Td[K];
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  double s1[NV], s2[NV], mx[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) s1[v] = s2[v] = mx[v] = 0.0;
  if (gi < A.nx && gj < A.ny) {
    const long long cell = (long long)gj * A.pitch + gi;
    const double area = (A.dx * A.dy) * 0.25;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double md[NB];
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        long long e = (long long)(v * NB + m) * A.plane + cell;
        md[m] = a[e] - (b ? b[e] : 0.0);
      }
      double acc1 = 0.0, acc2 = 0.0;
#pragma unroll
      for (int qa = 0; qa < NQ; ++qa)
#pragma unroll
        for (int qb = 0; qb < NQ; ++qb) {
          double d = 0.0;
#pragma unroll
          for (int m = 0; m < NB; ++m)
            d += md[m] * T.B[mode_deg(K, BASIS, m, 0)][qa] * T.B[mode_deg(K, BASIS, m, 1)][qb];
          double ww = T.wq[qa] * T.wq[qb];
          acc1 += fabs(d) * ww;
          acc2 += d * d * ww;
          mx[v] = fmax(mx[v], fabs(d));
        }
      s1[v] = acc1 * area;
      s2[v] = acc2 * area;
    }
  }
  // fixed-order tree reduction in shared memory (nthr <= 64 * 32 is not needed: nthr <= 1024)
  for (int k = 0; k < NV * 3; ++k) {
    double val = k < NV ? s1[k] : (k < 2 * NV ? s2[k - NV] : mx[k - 2 * NV]);
    bool ismax = k >= 2 * NV;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double other = __shfl_down_sync(0xffffffffu, val, o);
      val = ismax ? fmax(val, other) : val + other;
    }
    if ((tid & 31) == 0) red[k][tid >> 5] = val;
  }
  __syncthreads();
  if (tid < NV * 3) {
    int k = tid;
    bool ismax = k >= 2 * NV;
    double val = 0.0;
    for (int w = 0; w < (nthr + 31) / 32; ++w) val = ismax ? fmax(val, red[k][w]) : val + red[k][w];
    int blk = blockIdx.y * gridDim.x + blockIdx.x;
    partial[(long long)blk * NV * 3 + k] = val;
  }
}

static __global__ void k_norms_final(const double *partial, int nblk, double *out) {
  // one block of 12 threads: thread k reduces column k in block order (deterministic)
  int k = threadIdx.x;
  if (k >= NV * 3) return;
  bool ismax = k >= 2 * NV;
  double val = 0.0;
  for (int b = 0; b < nblk; ++b) {
    double x = partial[(long long)b * NV * 3 + k];
    val = ismax ? fmax(val, x) : val + x;
  }
  out[k] = val;
}

// FP64 cell-mean integrals of the full conserved state (equilibrium + perturbation),
// per-block partials [block][v] reduced by k_norms_final-style column sums.
template <typename R, int K, int BASIS>
__global__ void k_sums(const __grid_constant__ AuxArgs A, const Tab1D<double> *Td, const R *u,
                       double *partial) {
  constexpr int NB = num_modes(K, BASIS), NQ = K + 1;
  __shared__ double red[NV][64];
  const Tab1D<double> &T = Td[K];
  int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
  int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  double s[NV] = {0.0, 0.0, 0.0, 0.0};
  if (gi < A.nx && gj < A.ny) {
    const long long cell = (long long)gj * A.pitch + gi;
    double rbar = 0.0, pbar = 0.0;
    for (int qa = 0; qa < NQ; ++qa)
      for (int qb = 0; qb < NQ; ++qb) {
        double re, pe;
        eq_point64(A, A.fxv[gi * NQ + qa], A.fyv[gj * NQ + qb], re, pe);
        double ww = 0.25 * T.wq[qa] * T.wq[qb];
        rbar += re * ww;
        pbar += pe * ww;
      }
    double area = A.dx * A.dy;
    s[0] = (rbar + (double)u[(long long)(0 * NB) * A.plane + cell]) * area;
    s[1] = (double)u[(long long)(1 * NB) * A.plane + cell] * area;
    s[2] = (double)u[(long long)(2 * NB) * A.plane + cell] * area;
    s[3] = (pbar / (A.gamma - 1.0) + (double)u[(long long)(3 * NB) * A.plane + cell]) * area;
  }
  for (int k = 0; k < NV; ++k) {
    double val = s[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) val += __shfl_down_sync(0xffffffffu, val, o);
    if ((tid & 31) == 0) red[k][tid >> 5] = val;
  }
  __syncthreads();
  if (tid < NV) {
    double val = 0.0;
    for (int w = 0; w < (nthr + 31) / 32; ++w) val += red[tid][w];
    int blk = blockIdx.y * gridDim.x + blockIdx.x;
    partial[(long long)blk * NV + tid] = val;
  }
}

static __global__ void k_sums_final(const double *partial, int nblk, double *out) {
  int k = threadIdx.x;
  if (k >= NV) return;
  double val = 0.0;
  for (int b = 0; b < nblk; ++b) val += partial[(long long)b * NV + k];
  out[k] = val;
}

}  // namespace wb
