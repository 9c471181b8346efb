// wb_tables.cpp -- host-side basis, quadrature and equilibrium tables.
//
// The basis is the scaled Legendre family phi_a = sqrt(2a+1) P_a of 2d/legendre.f90:1-50
// with (k+1)-point Gauss-Legendre quadrature (2d/legendre.f90:77-108 computes it by Newton
// iteration).  The kernels' tables are the exact values of gen_ctab.py (wb_ctab.h);
// gauss_legendre / legendre_scaled below evaluate the same family at run time (Newton from
// the Chebyshev-node guess, Bonnet recurrence) for other uses.
#include "wb_tables.h"

#include "wb_ctab.h"

#include <cmath>

namespace wb {

void legendre_scaled(double x, int amax, double *phi, double *dphi) {
  double p[8], dp[8];
  p[0] = 1.0;
  dp[0] = 0.0;
  if (amax >= 1) {
    p[1] = x;
    dp[1] = 1.0;
  }
  for (int n = 1; n < amax; ++n) {
    p[n + 1] = ((2.0 * n + 1.0) * x * p[n] - n * p[n - 1]) / (n + 1.0);
    dp[n + 1] = dp[n - 1] + (2.0 * n + 1.0) * p[n];
  }
  for (int a = 0; a <= amax; ++a) {
    double s = std::sqrt(2.0 * a + 1.0);
    phi[a] = s * p[a];
    if (dphi) dphi[a] = s * dp[a];
  }
}

void gauss_legendre(int n, double *x, double *w) {
  const double pi = std::acos(-1.0);
  for (int i = 0; i < n; ++i) {
    // i-th largest root, refined by Newton on P_n
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double phi[8], dphi[8];
      legendre_scaled(z, n, phi, dphi);
      double s = std::sqrt(2.0 * n + 1.0);
      double dz = (phi[n] / s) / (dphi[n] / s);
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double phi[8], dphi[8];
    legendre_scaled(z, n, phi, dphi);
    double d = dphi[n] / std::sqrt(2.0 * n + 1.0);
    x[i] = -z;  // z runs from the largest root down, so x ascends
    w[i] = 2.0 / ((1.0 - z * z) * d * d);
  }
  // exact symmetry (x ascending: x[i] < 0 < x[n-1-i])
  for (int i = 0; i < n / 2; ++i) {
    double xm = 0.5 * (x[n - 1 - i] - x[i]), wm = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = -xm;
    x[n - 1 - i] = xm;
    w[i] = w[n - 1 - i] = wm;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// The tables every kernel uses come from the generated compile-time constants of
// wb_ctab.h (exact values rounded once), so the stage kernels (which fold them in as
// immediates) and the auxiliary kernels (which read them from constant memory) agree to
// the last bit.
template <int K>
static void fill_tab(Tab1D<double> &t) {
  for (int a = 0; a < NQMAX; ++a) {
    t.xq[a] = t.wq[a] = t.Ep[a] = t.Em[a] = 0.0;
    for (int q = 0; q < NQMAX; ++q) t.B[a][q] = t.D[a][q] = t.BW[a][q] = t.DW[a][q] = 0.0;
  }
  for (int q = 0; q <= K; ++q) {
    t.xq[q] = CTab<K>::xq(q);
    t.wq[q] = CTab<K>::wq(q);
    for (int a = 0; a <= K; ++a) {
      t.B[a][q] = CTab<K>::B(a, q);
      t.D[a][q] = CTab<K>::D(a, q);
      t.BW[a][q] = CTab<K>::BW(a, q);
      t.DW[a][q] = CTab<K>::DW(a, q);
    }
  }
  for (int a = 0; a <= K; ++a) {
    t.Ep[a] = CTab<K>::Ep(a);
    t.Em[a] = CTab<K>::Em(a);
  }
}

void make_tab1d(Tab1D<double> tabs[KMAX + 1]) {
  static_assert(KMAX == 2, "tables generated for degrees 0..2");
  fill_tab<0>(tabs[0]);
  fill_tab<1>(tabs[1]);
  fill_tab<2>(tabs[2]);
}

template <typename R>
void convert_tabs(const Tab1D<double> *in, Tab1D<R> *out, int n) {
  for (int k = 0; k < n; ++k) {
    for (int a = 0; a < NQMAX; ++a) {
      out[k].xq[a] = (R)in[k].xq[a];
      out[k].wq[a] = (R)in[k].wq[a];
      out[k].Ep[a] = (R)in[k].Ep[a];
      out[k].Em[a] = (R)in[k].Em[a];
      for (int q = 0; q < NQMAX; ++q) {
        out[k].B[a][q] = (R)in[k].B[a][q];
        out[k].D[a][q] = (R)in[k].D[a][q];
        out[k].BW[a][q] = (R)in[k].BW[a][q];
        out[k].DW[a][q] = (R)in[k].DW[a][q];
      }
    }
  }
}
template void convert_tabs<float>(const Tab1D<double> *, Tab1D<float> *, int);
template void convert_tabs<double>(const Tab1D<double> *, Tab1D<double> *, int);

double eq_factor_x(const EqParams &e, double x) {
  if (e.kind == 1) return std::exp(-(e.rho0 / e.p0) * e.gx * x);
  if (e.kind == 2) return 1.0 - (e.gamma - 1.0) / (e.gamma * e.kpoly) * e.gx * x;
  return 0.0;
}
double eq_factor_y(const EqParams &e, double y) {
  if (e.kind == 1) return std::exp(-(e.rho0 / e.p0) * e.gy * y);
  if (e.kind == 2) return -((e.gamma - 1.0) / (e.gamma * e.kpoly)) * e.gy * y;
  return 0.0;
}
void eq_combine(const EqParams &e, double fx, double fy, double *rho, double *p) {
  if (e.kind == 1) {
    double t = fx * fy;
    *rho = e.rho0 * t;
    *p = e.p0 * t;
  } else if (e.kind == 2) {
    double s = fx + fy;
    *rho = std::pow(s, 1.0 / (e.gamma - 1.0));
    *p = e.kpoly * (*rho * s);
  } else {
    *rho = 0.0;
    *p = 0.0;
  }
}

void make_eq_tables(const EqParams &e, int nx, int ny, double lx, double ly, int nq,
                    const double *xq, std::vector<double> &fxv, std::vector<double> &fxf,
                    std::vector<double> &fyv, std::vector<double> &fyf) {
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  fxv.assign((size_t)nx * nq, 0.0);
  fyv.assign((size_t)ny * nq, 0.0);
  fxf.assign((size_t)nx + 1, 0.0);
  fyf.assign((size_t)ny + 1, 0.0);
  for (int i = 0; i < nx; ++i)
    for (int q = 0; q < nq; ++q)
      fxv[(size_t)i * nq + q] = eq_factor_x(e, ((double)i + 0.5) * dx + dx / 2.0 * xq[q]);
  for (int j = 0; j < ny; ++j)
    for (int q = 0; q < nq; ++q)
      fyv[(size_t)j * nq + q] = eq_factor_y(e, ((double)j + 0.5) * dy + dy / 2.0 * xq[q]);
  for (int i = 0; i <= nx; ++i) fxf[i] = eq_factor_x(e, (double)i * dx);
  for (int j = 0; j <= ny; ++j) fyf[j] = eq_factor_y(e, (double)j * dy);
}

}  // namespace wb
