// wb_types.h -- types shared by the host layer and the sm_103a kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace wb {

constexpr int NV = 4;      // conserved variables (rho, mx, my, E)
constexpr int KMAX = 2;    // highest polynomial degree compiled
constexpr int NQMAX = KMAX + 1;

// Modes per variable for degree k and basis (0 = tensor Q_k, 1 = total degree P_k).
__host__ __device__ constexpr int num_modes(int k, int basis) {
  return basis == 0 ? (k + 1) * (k + 1) : (k + 1) * (k + 2) / 2;
}
// Mode m -> (a, b) in graded order (total degree, then a descending).
__host__ __device__ constexpr int mode_deg(int k, int basis, int m, int which) {
  int n = 0;
  int dmax = basis == 0 ? 2 * k : k;
  for (int d = 0; d <= dmax; ++d)
    for (int a = d; a >= 0; --a) {
      int b = d - a;
      if (a <= k && b <= k) {
        if (n == m) return which == 0 ? a : b;
        ++n;
      }
    }
  return -1;
}
__host__ __device__ constexpr int mode_index(int k, int basis, int a, int b) {
  int n = 0;
  int dmax = basis == 0 ? 2 * k : k;
  for (int d = 0; d <= dmax; ++d)
    for (int aa = d; aa >= 0; --aa) {
      int bb = d - aa;
      if (aa <= k && bb <= k) {
        if (aa == a && bb == b) return n;
        ++n;
      }
    }
  return -1;
}

// One-dimensional Gauss-Legendre tables for nq = k+1 points, basis
// phi_a = sqrt(2a+1) P_a.  B = phi_a(xi_q), D = phi_a'(xi_q), BW = B*w, DW = D*w,
// Ep/Em = phi_a(+1)/phi_a(-1).
template <typename R>
struct Tab1D {
  R xq[NQMAX], wq[NQMAX];
  R B[NQMAX][NQMAX], D[NQMAX][NQMAX], BW[NQMAX][NQMAX], DW[NQMAX][NQMAX];
  R Ep[NQMAX], Em[NQMAX];
};

// Device-resident run state: simulated time, step count, the fused wave-speed maxima
// (non-negative doubles stored as their bit patterns so atomicMax orders them) and
// the non-physical-state flag.  Double-buffered by step parity.
struct DevState {
  double t[2];
  unsigned long long smax[2][2];  // [parity][direction]
  long long nstep[2];
  double dt[2];  // batched form: the time step of the step that starts at parity p
  int err;  // bit 0: non-physical cell mean; bit 1: a bounded device wait gave up
  int pad;
};

// One output of a stage: out = sum_i c_i * [lim](in_i) + beta * Y + cdt * dt * L(Y).
template <typename R>
struct Combo {
  R *out;
  const R *in[2];
  R c[2];
  int lim[2];
  R beta, cdt;
};

// Compile-time variants of the stage kernel (bit mask).
constexpr int WB_VAR_POSITIVITY = 1;  // Zhang-Shu positivity limiter (limiter 2)
constexpr int WB_VAR_HLLC = 2;        // HLLC face flux instead of LLF

// 16-byte aligned (and sized): the batched form copies it into shared memory in 16-byte
// chunks.
template <typename R>
struct alignas(16) StageArgs {
  const R *x;                 // stage input (loaded with halo, limited if lim_y)
  Combo<R> o[2];              // o[1].out may be null
  int nx, ny;
  int pitch;                  // elements between rows of a plane (>= nx): cell (i, j) at j*pitch + i
  long long plane;            // elements between (var, mode) planes
  int bc_x, bc_y, llf_speed, limiter, lim_y;  // limiter: 0 off, 1 minmod, 2 positivity
  int riemann;                // 0 LLF, 1 HLLC (the kernel variant must match)
  int use_tma;                // interior tiles staged by one TMA copy (tensor map given)
  int eq_kind;
  R dx, dy, hidx, hidy;       // hidx = 0.5/dx, hidy = 0.5/dy
  R gamma, gm1, igm1, hgam;   // hgam = gamma/(gamma-1)
  R gx, gy;
  R rho0, p0, kpoly, npoly;   // npoly = 1/(gamma-1)
  R lim_norm, lim_Mdx2, lim_Mdy2, lim_tol;
  R lim_inorm;                // 1 / lim_norm (the limited slope is scaled back by a product)
  R pos_eps;                  // positivity limiter floor (limiter 2)
  // separable equilibrium factors: x at volume points [nx*nq], x at faces [nx+1], y likewise
  const R *fxv, *fxf, *fyv, *fyf;
  // time step
  int dt_mode;                // 0 fixed dt_fixed, 1 CFL from dev->smax[parity]
  int parity;
  int advance_time;           // first stage of a step: t[parity^1] = t[parity] + dt
  int compute_speed;          // last stage of a step: accumulate smax[parity^1]
  double dt_fixed;
  double cfl_over;            // cfl / (2k+1)
  double tend;                // > 0: clip dt at tend - t
  double ddx, ddy;            // dx, dy in double
  DevState *dev;
};

// Layout of one staged tile in shared memory (offsets in elements).  Rows are stored with
// pitch PX = TX + 8 starting at global column i0 - 4, so an x-interior row is one aligned
// run of 16-byte chunks:
//   su  [NV*NB][RY][PX]  modes of the tile and a one-cell halo (ring column rx at rx + 3);
//                        with the minmod limiter the columns of the second ring (i0 - 2 and
//                        i0 + TX + 1, stored at 2 and TX + 5) are staged too
//   sm  [NV][2][PX]      minmod limiter only: the means (mode 0) of rows j0 - 2 and
//                        j0 + TY + 1 over the ring-1 columns (stored at 3 .. TX + 4); with
//                        the mode-0 planes of su these are every neighbour mean the limiter
//                        of the one-cell ring reads
//   eq  fxv[NQ*(TX+2)], fxf[TX+1], fyv[NQ*(TY+2)], fyf[TY+1]  equilibrium factors (the
//       volume-point factors cover the one-cell halo, for the positivity limiter)
struct TileLayout {
  int TX, TY, RX, RY, PX, RXY, NB, NQ, lim;
  int su, sm, eq, buf;
};
__host__ __device__ inline TileLayout tile_layout(int K, int basis, int TX, int TY, int lim) {
  TileLayout L;
  L.TX = TX;
  L.TY = TY;
  L.RX = TX + 2;
  L.RY = TY + 2;
  L.PX = TX + 8;
  L.RXY = L.PX * L.RY;
  L.NB = num_modes(K, basis);
  L.NQ = K + 1;
  L.lim = lim;
  L.su = 0;
  L.sm = NV * L.NB * L.RXY;
  L.eq = L.sm + (lim ? NV * 2 * L.PX : 0);
  const int neq = L.NQ * (TX + 2) + TX + 1 + L.NQ * (TY + 2) + TY + 1;
  L.buf = (L.eq + neq + 31) & ~31;  // 128-byte aligned double buffers (TMA destinations)
  return L;
}

// Shared-memory bytes of the stage kernel for a TX x TY tile: reduction scratch, two
// staged tiles, and the x/y face fluxes of one tile.
template <typename R>
__host__ __device__ inline size_t stage_smem_bytes(int K, int basis, int TX, int TY, int lim) {
  const TileLayout L = tile_layout(K, basis, TX, TY, lim);
  const size_t flux = (size_t)NV * (K + 1) * ((size_t)TY * (TX + 1) + (size_t)(TY + 1) * TX);
  return 64 * sizeof(double) + (2 * (size_t)L.buf + flux) * sizeof(R);
}

// Arguments of the per-cell auxiliary kernels (FP64 equilibrium factors).
struct AuxArgs {
  int nx, ny;
  int pitch;  // elements between rows of a plane (>= nx)
  long long plane;
  int bc_x, bc_y, limiter, eq_kind;
  double dx, dy, gamma, gx, gy, rho0, p0, kpoly, npoly;
  double lim_norm, lim_Mdx2, lim_Mdy2, lim_tol;
  const double *fxv, *fxf, *fyv, *fyf;  // FP64 separable equilibrium factors
};

// Seeded perturbation (initial condition) parameters.
struct IcArgs {
  int kind, nmodes;
  double amp, xc, yc, sigma;
  double kx[32], ky[32], pu[32], pv[32], wt[32];
};

}  // namespace wb
