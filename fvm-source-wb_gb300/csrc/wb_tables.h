// wb_tables.h -- host-side basis, quadrature and equilibrium tables.
#pragma once
#include <vector>
#include "wb_types.h"

namespace wb {

// Gauss-Legendre nodes (ascending) and weights on [-1,1] for n points.
void gauss_legendre(int n, double *x, double *w);
// phi_a = sqrt(2a+1) P_a and its derivative at x, for a = 0..amax.
void legendre_scaled(double x, int amax, double *phi, double *dphi);
// Tables for degrees 0..KMAX (entry k has k+1 points).
void make_tab1d(Tab1D<double> tabs[KMAX + 1]);
template <typename R>
void convert_tabs(const Tab1D<double> *in, Tab1D<R> *out, int n);

struct EqParams {
  int kind;  // 0 none, 1 isothermal, 2 polytrope
  double gamma, gx, gy, rho0, p0, kpoly;
};
// Separable equilibrium factors: isothermal fx = exp(-(rho0/p0) gx x),
// polytrope fx = 1 - (gamma-1)/(gamma K) gx x (and fy = -(gamma-1)/(gamma K) gy y).
double eq_factor_x(const EqParams &e, double x);
double eq_factor_y(const EqParams &e, double y);
// density and pressure from the two factors
void eq_combine(const EqParams &e, double fx, double fy, double *rho, double *p);

// Factor tables of an nx x ny grid on [0,lx]x[0,ly] with nq points per direction:
// fxv[i*nq+q] at volume points, fxf[i] at the nx+1 x-faces; likewise y.
void make_eq_tables(const EqParams &e, int nx, int ny, double lx, double ly, int nq,
                    const double *xq, std::vector<double> &fxv, std::vector<double> &fxf,
                    std::vector<double> &fyv, std::vector<double> &fyf);

// The reference's snapshot number format, Fortran 1PE12.5 (12 columns, E+dd, or +ddd with
// the E dropped for three-digit exponents), into out[16]; and its reader.
void fortran_1pe12_5(double v, char *out);
bool parse_fortran_real(const char *tok, double *v);

}  // namespace wb
