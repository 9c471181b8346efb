/*
 * wb_oracle.c -- CPU restatement (FP64) of the reference's well-balanced
 * Euler-with-gravity step.  TEST INFRASTRUCTURE ONLY: the parity checker for the
 * CUDA path and the timed CPU baseline; never linked into the product library.
 *
 * Parity status: see wb_oracle.h (basis KAT-pinned, operator parity unpinned).
 *
 * Every routine cites the reference file:line it restates.  Loop orders follow the
 * reference where the reference defines them, so summations round the same way.
 * Reference defects are reproduced only where a flag says so (orc_ref2d_*).
 */
#include "wb_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV 4
#define KMAX 3
#define NQMAX (KMAX + 1)
#define NBMAX ((KMAX + 1) * (KMAX + 1))

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }

/* compute_primitive floors rho with the default-real literal 10e-10
 * (2d/benchmark_2d_dg.f90:898); compute_speed floors with 1d-10 (:885). */
static const double PRIM_RHO_FLOOR = (double)1.0e-9f;
static const double SPEED_FLOOR = 1e-10;

/* ------------------------------------------------------------------ basis */

/* 2d/legendre.f90:1-25: phi_n(x) = sqrt(2n+1) P_n(x), x clamped to [-1,1] */
double orc_legendre(double x, int n) {
  double p = 0.0;
  x = fmin(fmax(x, -1.0), 1.0);
  switch (n) {
  case 0: p = 1.0; break;
  case 1: p = x; break;
  case 2: p = 0.5 * (3 * (x * x) - 1); break;
  case 3: p = 0.5 * (5.0 * (x * x * x) - 3.0 * x); break;
  case 4: p = 0.125 * (35.0 * ((x * x) * (x * x)) - 30.0 * (x * x) + 3.0); break;
  case 5: p = 0.125 * (63.0 * ((x * x) * (x * x) * x) - 70.0 * (x * x * x) + 15.0 * x); break;
  case 6:
    p = 1.0 / 16.0 * (231.0 * ((x * x * x) * (x * x * x)) - 315.0 * ((x * x) * (x * x)) +
                      105.0 * (x * x) - 5.0);
    break;
  }
  return sqrt((2.0 * (double)n + 1.0)) * p;
}

/* 2d/legendre.f90:27-50 */
double orc_legendre_prime(double x, int n) {
  double p = 0.0;
  x = fmin(fmax(x, -1.0), 1.0);
  switch (n) {
  case 0: p = 0.0; break;
  case 1: p = 1.0; break;
  case 2: p = 3.0 * x; break;
  case 3: p = 0.5 * (15.0 * (x * x) - 3.0); break;
  case 4: p = 0.125 * (140.0 * (x * x * x) - 60.0 * x); break;
  case 5: p = 0.125 * (315.0 * ((x * x) * (x * x)) - 210.0 * (x * x) + 15.0); break;
  case 6:
    p = 1.0 / 16.0 * (1386.0 * ((x * x) * (x * x) * x) - 1260.0 * (x * x * x) + 210.0 * x);
    break;
  }
  return sqrt((2.0 * (double)n + 1.0)) * p;
}

/* 2d/legendre.f90:77-108: Newton iteration (500 steps) from the Tricomi-type guess;
 * the guess prefactor is evaluated in default (single) real as in the reference. */
void orc_gl_quadrature(int n, double *xq, double *wq) {
  const double dpi = acos(-1.0);
  for (int i = 1; i <= n; ++i) {
    float fn = (float)n;
    float g = 1.0f - 0.125f / fn / fn + 0.125f / fn / fn / fn;
    double xx = (double)g * cos(dpi * (4.0 * (double)i - 1.0) / (4.0 * (double)n + 2.0));
    for (int it = 0; it < 500; ++it) xx = xx - orc_legendre(xx, n) / orc_legendre_prime(xx, n);
    xq[i - 1] = -xx;
    double lp = orc_legendre_prime(xq[i - 1], n);
    wq[i - 1] = 2 * (2.0 * (double)n + 1.0) / (1.0 - xq[i - 1] * xq[i - 1]) / (lp * lp);
  }
  for (int i = n / 2 + 1; i <= n; ++i) {
    xq[i - 1] = -xq[n - i];
    wq[i - 1] = wq[n - i];
  }
}

/* Mode list.  Q_k: all (a,b) with a,b <= k (the reference's mx*my modes,
 * 2d/benchmark_2d_dg.f90:1217-1242); P_k: a+b <= k.  Graded order: total degree d,
 * then a descending. */
int orc_modes(int k, int basis, int *ma, int *mb) {
  int n = 0, dmax = basis == ORC_BASIS_Q ? 2 * k : k;
  for (int d = 0; d <= dmax; ++d)
    for (int a = d; a >= 0; --a) {
      int b = d - a;
      if (a <= k && b <= k) {
        if (ma) ma[n] = a;
        if (mb) mb[n] = b;
        ++n;
      }
    }
  return n;
}
int orc_nb(int k, int basis) { return orc_modes(k, basis, NULL, NULL); }

typedef struct {
  int k, nq, nb;
  int ma[NBMAX], mb[NBMAX];
  int idx[NQMAX][NQMAX];   /* (a,b) -> mode index or -1 */
  double xq[NQMAX], wq[NQMAX];
  double B[NQMAX][NQMAX];  /* phi_a(xi_q) */
  double D[NQMAX][NQMAX];  /* phi_a'(xi_q) */
  double Ep[NQMAX], Em[NQMAX]; /* phi_a(+1), phi_a(-1) */
  double dx, dy;
} tabs_t;

static void make_tabs(const orc_cfg *c, tabs_t *t) {
  memset(t, 0, sizeof(*t));
  t->k = c->order;
  t->nq = c->order + 1;
  t->nb = orc_modes(c->order, c->basis, t->ma, t->mb);
  for (int a = 0; a < NQMAX; ++a)
    for (int b = 0; b < NQMAX; ++b) t->idx[a][b] = -1;
  for (int m = 0; m < t->nb; ++m) t->idx[t->ma[m]][t->mb[m]] = m;
  orc_gl_quadrature(t->nq, t->xq, t->wq);
  for (int a = 0; a < t->nq; ++a) {
    for (int q = 0; q < t->nq; ++q) {
      t->B[a][q] = orc_legendre(t->xq[q], a);
      t->D[a][q] = orc_legendre_prime(t->xq[q], a);
    }
    t->Ep[a] = orc_legendre(1.0, a);
    t->Em[a] = orc_legendre(-1.0, a);
  }
  t->dx = c->lx / (double)c->nx;
  t->dy = c->ly / (double)c->ny;
}

/* quadrature-point coordinates, 2d/benchmark_2d_dg.f90:112-113 (0-based cell i) */
static inline double xvol(const tabs_t *t, int i, int q) {
  return ((double)i + 0.5) * t->dx + t->dx / 2.0 * t->xq[q];
}
static inline double yvol(const tabs_t *t, int j, int q) {
  return ((double)j + 0.5) * t->dy + t->dy / 2.0 * t->xq[q];
}
/* face coordinates, benchmark_2d.f90:498-508 */
static inline double xface(const tabs_t *t, int i) { return (double)i * t->dx; }
static inline double yface(const tabs_t *t, int j) { return (double)j * t->dy; }

/* ------------------------------------------------------------ equilibrium */

/* Separable factors of the equilibrium for a linear potential Phi = gx x + gy y.
 * Isothermal (2d/benchmark_2d_dg.f90:605-615, benchmark_1d.f90:138-146):
 *   rho = rho0 * (fx*fy), p = p0 * (fx*fy), fx = exp(-kappa gx x), fy = exp(-kappa gy y),
 *   kappa = rho0/p0.
 * Polytrope (benchmark_1d.f90:59-61,149-151, generalised to K):
 *   s = fx + fy, fx = 1 - c gx x, fy = -c gy y, c = (gamma-1)/(gamma K),
 *   rho = s^(1/(gamma-1)), p = K * (rho*s)  (= K rho^gamma). */
static double eq_fx(const orc_cfg *c, double x) {
  if (c->eq_kind == ORC_EQ_ISOTHERMAL) return exp(-(c->rho0 / c->p0) * c->gx * x);
  if (c->eq_kind == ORC_EQ_POLYTROPE)
    return 1.0 - (c->gamma - 1.0) / (c->gamma * c->kpoly) * c->gx * x;
  return 0.0;
}
static double eq_fy(const orc_cfg *c, double y) {
  if (c->eq_kind == ORC_EQ_ISOTHERMAL) return exp(-(c->rho0 / c->p0) * c->gy * y);
  if (c->eq_kind == ORC_EQ_POLYTROPE)
    return -((c->gamma - 1.0) / (c->gamma * c->kpoly)) * c->gy * y;
  return 0.0;
}
void orc_eq_point(const orc_cfg *c, double fx, double fy, double sx_unused, double sy_unused,
                  double *rho, double *p) {
  (void)sx_unused;
  (void)sy_unused;
  if (c->eq_kind == ORC_EQ_ISOTHERMAL) {
    double t = fx * fy;
    *rho = c->rho0 * t;
    *p = c->p0 * t;
  } else if (c->eq_kind == ORC_EQ_POLYTROPE) {
    double s = fx + fy;
    *rho = pow(s, 1.0 / (c->gamma - 1.0));
    *p = c->kpoly * (*rho * s);
  } else {
    *rho = 0.0;
    *p = 0.0;
  }
}
void orc_eq_at(const orc_cfg *c, double x, double y, double *rho, double *p) {
  orc_eq_point(c, eq_fx(c, x), eq_fy(c, y), 0, 0, rho, p);
}

/* -------------------------------------------------------------- physics */

/* compute_primitive, 2d/benchmark_2d_dg.f90:891-903 */
static inline void prim(double g, const double *u, double *w) {
  w[0] = fmax(u[0], PRIM_RHO_FLOOR);
  w[1] = u[1] / w[0];
  w[2] = u[2] / w[0];
  w[3] = (g - 1.0) * (u[3] - 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2]));
}
/* compute_flux_int, 2d/benchmark_2d_dg.f90:944-963 (dir 0 = x, 1 = y) */
static inline void flux_dir(const double *u, const double *w, int dir, double *f) {
  if (dir == 0) {
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
/* compute_speed sound speed, 2d/benchmark_2d_dg.f90:873-889 */
static inline double sound(double g, const double *w) {
  return sqrt(g * fmax(w[3], SPEED_FLOOR) / fmax(w[0], SPEED_FLOOR));
}
/* gravity source with the correct sign -rho grad(Phi), benchmark_2d.f90:327-350 */
static inline void source(const double *w, double gx, double gy, double *s) {
  s[0] = 0.0;
  s[1] = -(w[0] * gx);
  s[2] = -(w[0] * gy);
  s[3] = -(w[0] * (w[1] * gx + w[2] * gy));
}
/* compute_llflux, 2d/benchmark_2d_dg.f90:968-988 (ORC_LLF_REF2D), or the
 * max(|v_n|+c) estimate of benchmark_2d.f90:353-367 / dg_with_source.f90:1299-1316 */
static inline void llf(const orc_cfg *c, const double *uL, const double *uR, int dir,
                       double *fh) {
  double wL[NV], wR[NV], fL[NV], fR[NV];
  prim(c->gamma, uL, wL);
  prim(c->gamma, uR, wR);
  flux_dir(uL, wL, dir, fL);
  flux_dir(uR, wR, dir, fR);
  double cL = sound(c->gamma, wL), cR = sound(c->gamma, wR);
  double vL = wL[1 + dir], vR = wR[1 + dir], cmax;
  if (c->llf_speed == ORC_LLF_REF2D)
    cmax = fmax(fabs(vR + cR), fabs(vL + cL));
  else
    cmax = fmax(fabs(vL) + cL, fabs(vR) + cR);
  for (int v = 0; v < NV; ++v) fh[v] = 0.5 * (fR[v] + fL[v]) + 0.5 * cmax * (uL[v] - uR[v]);
}

/* HLLC (riemann = 2 of dg_with_source.f90; riemann_hllc :1318-1374) for 2D states, the
 * transverse velocity carried by the contact.  Davis wave speeds S_L = min(v_L, v_R) -
 * max(c_L, c_R), S_R = max(v_L, v_R) + max(c_L, c_R) (:1332-1333), contact speed from the
 * Lagrangian speeds D_L = rho_L (v_L - S_L), D_R = rho_R (S_R - v_R) (:1335-1338), sampled
 * at x/t = 0 in the order of :1346-1366.  The star fluxes are written F_K + S_K (U*_K - U_K)
 * with U*_K - U_K = (S* - v_K)/(S_K - S*) [rho_K, rho_K S_K, rho_K vt_K,
 * E_K + p_K + rho_K S* (S_K - v_K)], which equals riemann_hllc's F(U*_K) in exact arithmetic
 * and gives F(u) bit for bit when u_L = u_R at rest (S* = v_K = 0). */
static inline void hllc(const orc_cfg *c, const double *uL, const double *uR, int dir,
                        double *fh) {
  double wL[NV], wR[NV], fL[NV], fR[NV];
  prim(c->gamma, uL, wL);
  prim(c->gamma, uR, wR);
  flux_dir(uL, wL, dir, fL);
  flux_dir(uR, wR, dir, fR);
  const double cL = sound(c->gamma, wL), cR = sound(c->gamma, wR);
  const double vL = wL[1 + dir], vR = wR[1 + dir];
  const double SL = fmin(vL, vR) - fmax(cL, cR), SR = fmax(vL, vR) + fmax(cL, cR);
  const double DL = wL[0] * (vL - SL), DR = wR[0] * (SR - vR);
  const double Ss = (DR * vR + DL * vL + (wL[3] - wR[3])) / (DL + DR);
  const double *u, *w, *f;
  double SK;
  if (SL > 0.0) {
    for (int v = 0; v < NV; ++v) fh[v] = fL[v];
    return;
  } else if (Ss > 0.0) {
    u = uL; w = wL; f = fL; SK = SL;
  } else if (SR > 0.0) {
    u = uR; w = wR; f = fR; SK = SR;
  } else {
    for (int v = 0; v < NV; ++v) fh[v] = fR[v];
    return;
  }
  const double vK = w[1 + dir], q = SK * ((Ss - vK) / (SK - Ss));
  double d[NV];
  d[0] = w[0];
  d[1 + dir] = w[0] * SK;
  d[2 - dir] = w[0] * w[2 - dir];
  d[3] = (u[3] + w[3]) + w[0] * Ss * (SK - vK);
  for (int v = 0; v < NV; ++v) fh[v] = f[v] + q * d[v];
}

void orc_num_flux(const orc_cfg *c, const double *uL, const double *uR, int dir, double *f) {
  if (c->riemann == ORC_RIEMANN_HLLC) hllc(c, uL, uR, dir, f);
  else llf(c, uL, uR, dir, f);
}

/* BC index map, 2d/benchmark_2d_dg.f90:777-824 (bc=1 periodic, bc=2,3 copy) */
static inline int bcmap(int i, int n, int bc) {
  if (i < 0) return bc == ORC_BC_PERIODIC ? i + n : 0;
  if (i >= n) return bc == ORC_BC_PERIODIC ? i - n : n - 1;
  return i;
}

/* ---------------------------------------------------- modal <-> nodal */

/* get_nodes_from_modes, 2d/benchmark_2d_dg.f90:544-592: loops modes (a outer, b inner) */
void orc_nodes_from_modes(const orc_cfg *c, int nvar, const double *modes, double *nodes) {
  tabs_t t;
  make_tabs(c, &t);
  size_t nc = (size_t)c->nx * c->ny;
  int nq2 = t.nq * t.nq;
  for (int v = 0; v < nvar; ++v)
    for (size_t cell = 0; cell < nc; ++cell)
      for (int qa = 0; qa < t.nq; ++qa)
        for (int qb = 0; qb < t.nq; ++qb) {
          double s = 0.0;
          for (int a = 0; a < t.nq; ++a)
            for (int b = 0; b < t.nq; ++b) {
              int m = t.idx[a][b];
              if (m < 0) continue;
              s = s + modes[((size_t)v * t.nb + m) * nc + cell] * t.B[a][qa] * t.B[b][qb];
            }
          nodes[((size_t)v * nq2 + qa * t.nq + qb) * nc + cell] = s;
        }
}

/* get_modes_from_nodes, 2d/benchmark_2d_dg.f90:497-542 */
void orc_modes_from_nodes(const orc_cfg *c, int nvar, const double *nodes, double *modes) {
  tabs_t t;
  make_tabs(c, &t);
  size_t nc = (size_t)c->nx * c->ny;
  int nq2 = t.nq * t.nq;
  for (int v = 0; v < nvar; ++v)
    for (size_t cell = 0; cell < nc; ++cell)
      for (int m = 0; m < t.nb; ++m) {
        int a = t.ma[m], b = t.mb[m];
        double s = 0.0;
        for (int qa = 0; qa < t.nq; ++qa)
          for (int qb = 0; qb < t.nq; ++qb)
            s = s + 0.25 * nodes[((size_t)v * nq2 + qa * t.nq + qb) * nc + cell] * t.B[a][qa] *
                        t.B[b][qb] * t.wq[qa] * t.wq[qb];
        modes[((size_t)v * t.nb + m) * nc + cell] = s;
      }
}

/* ------------------------------------------------------------- seeding */

/* splitmix64 (Steele, Lea, Flood 2014) */
uint64_t orc_splitmix64(uint64_t *state) {
  uint64_t z = (*state += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
double orc_uniform(uint64_t *state) {
  return (double)(orc_splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

/* Perturbation at a point, in conservative variables (delta of rho, m_x, m_y, E).
 * Pressure bump: the hydrostatic IC of 2d/benchmark_2d_dg.f90:145-153 with its
 * Gaussian 'eta' term; velocity modes: u = v = 0 equilibrium plus a velocity field at
 * unchanged rho and p (compute_conservative, :905-917). */
static void ic_point(const orc_cfg *c, const orc_ic *ic, double x, double y, double rhoe,
                     double *d) {
  d[0] = d[1] = d[2] = d[3] = 0.0;
  if (ic->kind == 1) {
    double rx = x - ic->xc, ry = y - ic->yc;
    double dp = ic->amp * exp(-(rx * rx + ry * ry) / (2.0 * ic->sigma * ic->sigma));
    d[3] = dp * (1.0 / (c->gamma - 1.0));
  } else if (ic->kind == 2) {
    const double tpi = 2.0 * acos(-1.0);
    double du = 0.0, dv = 0.0;
    for (int m = 0; m < ic->nmodes; ++m) {
      double arg = tpi * (ic->kx[m] * x + ic->ky[m] * y);
      du += ic->weight[m] * sin(arg + ic->phase_u[m]);
      dv += ic->weight[m] * sin(arg + ic->phase_v[m]);
    }
    du *= ic->amp;
    dv *= ic->amp;
    d[1] = rhoe * du;
    d[2] = rhoe * dv;
    d[3] = 0.5 * rhoe * (du * du + dv * dv);
  }
}

/* IC projection onto modes, as get_modes_from_nodes (2d/benchmark_2d_dg.f90:497-542) */
void orc_project_ic(const orc_cfg *c, const orc_ic *ic, double *delta) {
  tabs_t t;
  make_tabs(c, &t);
  size_t nc = (size_t)c->nx * c->ny;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 0; j < c->ny; ++j)
    for (int i = 0; i < c->nx; ++i) {
      size_t cell = (size_t)j * c->nx + i;
      double dq[NQMAX][NQMAX][NV];
      for (int qa = 0; qa < t.nq; ++qa)
        for (int qb = 0; qb < t.nq; ++qb) {
          double x = xvol(&t, i, qa), y = yvol(&t, j, qb), re, pe;
          orc_eq_point(c, eq_fx(c, x), eq_fy(c, y), 0, 0, &re, &pe);
          ic_point(c, ic, x, y, re, dq[qa][qb]);
        }
      for (int v = 0; v < NV; ++v)
        for (int m = 0; m < t.nb; ++m) {
          int a = t.ma[m], b = t.mb[m];
          double s = 0.0;
          for (int qa = 0; qa < t.nq; ++qa)
            for (int qb = 0; qb < t.nq; ++qb)
              s = s + 0.25 * dq[qa][qb][v] * t.B[a][qa] * t.B[b][qb] * t.wq[qa] * t.wq[qb];
          delta[((size_t)v * t.nb + m) * nc + cell] = s;
        }
    }
}

/* ------------------------------------------- the 2D well-balanced operator */

/* Trace of cell `cell` at reference point (xi, eta) given by basis values
 * pa[a] = phi_a(xi), pb[b] = phi_b(eta); modes summed a outer, b inner as
 * 2d/benchmark_2d_dg.f90:1258-1268. */
static inline void trace(const tabs_t *t, const double *u, size_t nc, size_t cell,
                         const double *pa, const double *pb, double *d) {
  for (int v = 0; v < NV; ++v) {
    double s = 0.0;
    for (int a = 0; a < t->nq; ++a)
      for (int b = 0; b < t->nq; ++b) {
        int m = t->idx[a][b];
        if (m < 0) continue;
        s = s + u[((size_t)v * t->nb + m) * nc + cell] * pa[a] * pb[b];
      }
    d[v] = s;
  }
}

/*
 * dudt = L(u_eq + delta) - L(u_eq), the delta-split of
 * dg_with_source.f90:1749-2031 (compute_update_exact_delta) applied pointwise to the
 * 2D modal DG operator of 2d/benchmark_2d_dg.f90:1137-1479:
 *   volume  :1207-1244  vol1 = sum F1 phi_a'(xi) w phi_b(eta) w, vol2 likewise with G
 *   traces  :1253-1314  delta at xi = +-1 on the GL eta points (and vice versa)
 *   faces   :1333-1366  LLF on (u_eq(face) + delta_L, u_eq(face) + delta_R), the face
 *                       equilibrium of benchmark_2d.f90:505-537
 *   edges   :1372-1411
 *   source  :1426-1443  S = -rho grad Phi (benchmark_2d.f90:337-345)
 *   assembly:1449-1466  0.5*(vol - edges)/dx,dy + 0.25*source
 * At every volume/face point the flux and source of the equilibrium state are
 * subtracted from those of the perturbed state (F(u_eq+d) - F(u_eq)), so a zero
 * perturbation gives an exactly zero update.
 */
void orc_rhs(const orc_cfg *c, const double *delta, double *dudt) {
  tabs_t t;
  make_tabs(c, &t);
  const int nx = c->nx, ny = c->ny, nq = t.nq, nb = t.nb;
  const size_t nc = (size_t)nx * ny;
  const double g = c->gamma, igm1 = 1.0 / (c->gamma - 1.0);
  /* face fluxes: x-faces [(ny)][(nx+1)][NV][nq], y-faces [(ny+1)][nx][NV][nq] */
  double *Fx = (double *)malloc(sizeof(double) * (size_t)(nx + 1) * ny * NV * nq);
  double *Fy = (double *)malloc(sizeof(double) * (size_t)nx * (ny + 1) * NV * nq);

#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 0; j < ny; ++j)
    for (int fi = 0; fi <= nx; ++fi) {
      int il = bcmap(fi - 1, nx, c->bc_x), ir = bcmap(fi, nx, c->bc_x);
      size_t cl = (size_t)j * nx + il, cr = (size_t)j * nx + ir;
      double fxf = eq_fx(c, xface(&t, fi));
      for (int q = 0; q < nq; ++q) {
        double dL[NV], dR[NV], pb[NQMAX];
        for (int b = 0; b < nq; ++b) pb[b] = t.B[b][q];
        trace(&t, delta, nc, cl, t.Ep, pb, dL);
        trace(&t, delta, nc, cr, t.Em, pb, dR);
        double re, pe;
        orc_eq_point(c, fxf, eq_fy(c, yvol(&t, j, q)), 0, 0, &re, &pe);
        double ue[NV] = {re, 0.0, 0.0, pe * igm1}, uL[NV], uR[NV], fh[NV], we[NV], fe[NV];
        for (int v = 0; v < NV; ++v) {
          uL[v] = ue[v] + dL[v];
          uR[v] = ue[v] + dR[v];
        }
        orc_num_flux(c, uL, uR, 0, fh);
        prim(g, ue, we);
        flux_dir(ue, we, 0, fe);
        for (int v = 0; v < NV; ++v)
          Fx[(((size_t)j * (nx + 1) + fi) * NV + v) * nq + q] = fh[v] - fe[v];
      }
    }

#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int fj = 0; fj <= ny; ++fj)
    for (int i = 0; i < nx; ++i) {
      int jb = bcmap(fj - 1, ny, c->bc_y), jt = bcmap(fj, ny, c->bc_y);
      size_t cb = (size_t)jb * nx + i, ct = (size_t)jt * nx + i;
      double fyf = eq_fy(c, yface(&t, fj));
      for (int q = 0; q < nq; ++q) {
        double dB[NV], dT[NV], pa[NQMAX];
        for (int a = 0; a < nq; ++a) pa[a] = t.B[a][q];
        trace(&t, delta, nc, cb, pa, t.Ep, dB);
        trace(&t, delta, nc, ct, pa, t.Em, dT);
        double re, pe;
        orc_eq_point(c, eq_fx(c, xvol(&t, i, q)), fyf, 0, 0, &re, &pe);
        double ue[NV] = {re, 0.0, 0.0, pe * igm1}, uB[NV], uT[NV], fh[NV], we[NV], fe[NV];
        for (int v = 0; v < NV; ++v) {
          uB[v] = ue[v] + dB[v];
          uT[v] = ue[v] + dT[v];
        }
        orc_num_flux(c, uB, uT, 1, fh);
        prim(g, ue, we);
        flux_dir(ue, we, 1, fe);
        for (int v = 0; v < NV; ++v)
          Fy[(((size_t)fj * nx + i) * NV + v) * nq + q] = fh[v] - fe[v];
      }
    }

  const double idx = 1.0 / t.dx, idy = 1.0 / t.dy;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      size_t cell = (size_t)j * nx + i;
      double dF[NQMAX][NQMAX][NV], dG[NQMAX][NQMAX][NV], dS[NQMAX][NQMAX][NV];
      double fxv[NQMAX], fyv[NQMAX];
      for (int q = 0; q < nq; ++q) {
        fxv[q] = eq_fx(c, xvol(&t, i, q));
        fyv[q] = eq_fy(c, yvol(&t, j, q));
      }
      for (int qa = 0; qa < nq; ++qa)
        for (int qb = 0; qb < nq; ++qb) {
          double pa[NQMAX], pb[NQMAX], d[NV], re, pe;
          for (int a = 0; a < nq; ++a) {
            pa[a] = t.B[a][qa];
            pb[a] = t.B[a][qb];
          }
          trace(&t, delta, nc, cell, pa, pb, d);
          orc_eq_point(c, fxv[qa], fyv[qb], 0, 0, &re, &pe);
          double ue[NV] = {re, 0.0, 0.0, pe * igm1}, u[NV], w[NV], we[NV];
          double f[NV], fe[NV], gg[NV], ge[NV], s[NV], se[NV];
          for (int v = 0; v < NV; ++v) u[v] = ue[v] + d[v];
          prim(g, u, w);
          prim(g, ue, we);
          flux_dir(u, w, 0, f);
          flux_dir(ue, we, 0, fe);
          flux_dir(u, w, 1, gg);
          flux_dir(ue, we, 1, ge);
          source(w, c->gx, c->gy, s);
          source(we, c->gx, c->gy, se);
          for (int v = 0; v < NV; ++v) {
            dF[qa][qb][v] = f[v] - fe[v];
            dG[qa][qb][v] = gg[v] - ge[v];
            dS[qa][qb][v] = s[v] - se[v];
          }
        }
      for (int v = 0; v < NV; ++v)
        for (int m = 0; m < nb; ++m) {
          int a = t.ma[m], b = t.mb[m];
          double vol1 = 0.0, vol2 = 0.0, src = 0.0, e1 = 0.0, e2 = 0.0, e3 = 0.0, e4 = 0.0;
          for (int qa = 0; qa < nq; ++qa)
            for (int qb = 0; qb < nq; ++qb) {
              vol1 = vol1 + dF[qa][qb][v] * t.D[a][qa] * t.wq[qa] * t.B[b][qb] * t.wq[qb];
              vol2 = vol2 + dG[qa][qb][v] * t.D[b][qb] * t.wq[qb] * t.B[a][qa] * t.wq[qa];
              src = src + dS[qa][qb][v] * t.B[a][qa] * t.wq[qa] * t.B[b][qb] * t.wq[qb];
            }
          for (int q = 0; q < nq; ++q) {
            e1 = e1 + Fx[(((size_t)j * (nx + 1) + i + 1) * NV + v) * nq + q] * t.Ep[a] * t.B[b][q] *
                          t.wq[q];
            e2 = e2 + Fx[(((size_t)j * (nx + 1) + i) * NV + v) * nq + q] * t.Em[a] * t.B[b][q] *
                          t.wq[q];
            e3 = e3 + Fy[(((size_t)(j + 1) * nx + i) * NV + v) * nq + q] * t.Ep[b] * t.B[a][q] *
                          t.wq[q];
            e4 = e4 + Fy[(((size_t)j * nx + i) * NV + v) * nq + q] * t.Em[b] * t.B[a][q] * t.wq[q];
          }
          dudt[((size_t)v * nb + m) * nc + cell] =
              (idx * vol1 + idy * vol2 - idx * (e1 - e2) - idy * (e3 - e4)) / 2. + src / 4.;
        }
    }
  free(Fx);
  free(Fy);
}

/* minmod, 2d/limiters.f90:18-28 */
static inline double minmod3(double x, double y, double z) {
  double s = copysign(1.0, x);
  if (copysign(1.0, y) == s && copysign(1.0, z) == s) return s * fmin(fmin(fabs(x), fabs(y)), fabs(z));
  return 0.0;
}
/* generalized_minmod, 2d/limiters.f90:30-54 (M*dx^2 bypass; M=0 -> plain minmod) */
static inline double gminmod(double x, double y, double z, double M, double h) {
  if (fabs(x) < M * h * h) return x;
  return minmod3(x, y, z);
}

/*
 * Moment limiter on the perturbation, after compute_limiter (2d/limiters.f90:203-309):
 * first moments are limited against neighbour-mean differences with the norm=3
 * scaling (:224,254-260); a cell whose limited slopes differ from the old ones by
 * more than lim_tol (:262) gets the limited slopes and its higher modes dropped,
 * otherwise it is left untouched.  Applied to delta (conservative), not to primitive
 * modes, so the equilibrium is never limited (the rule of dg_with_source.f90:565-577).
 */
void orc_limit(const orc_cfg *c, const double *in, double *out) {
  tabs_t t;
  make_tabs(c, &t);
  const int nx = c->nx, ny = c->ny, nb = t.nb;
  const size_t nc = (size_t)nx * ny;
  if (c->limiter == 2) {
    orc_positivity(c, in, out);
    return;
  }
  memcpy(out, in, sizeof(double) * nc * NV * nb);
  if (c->limiter != 1 || c->order < 1) return;
  const int m10 = t.idx[1][0], m01 = t.idx[0][1];
  const double nrm = c->lim_norm;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      size_t cell = (size_t)j * nx + i;
      size_t cw = (size_t)j * nx + bcmap(i - 1, nx, c->bc_x);
      size_t ce = (size_t)j * nx + bcmap(i + 1, nx, c->bc_x);
      size_t cs = (size_t)bcmap(j - 1, ny, c->bc_y) * nx + i;
      size_t cn = (size_t)bcmap(j + 1, ny, c->bc_y) * nx + i;
      for (int v = 0; v < NV; ++v) {
        const double *u0 = in + (size_t)v * nb * nc;
        double m0 = u0[cell];
        double sx = in[((size_t)v * nb + m10) * nc + cell];
        double sy = in[((size_t)v * nb + m01) * nc + cell];
        double l1 = gminmod(nrm * sx, u0[ce] - m0, m0 - u0[cw], c->lim_M, t.dx) / nrm;
        double l2 = gminmod(nrm * sy, u0[cn] - m0, m0 - u0[cs], c->lim_M, t.dy) / nrm;
        if (fabs(l1 - sx) > c->lim_tol || fabs(l2 - sy) > c->lim_tol) {
          out[((size_t)v * nb + m10) * nc + cell] = l1;
          out[((size_t)v * nb + m01) * nc + cell] = l2;
          for (int m = 0; m < nb; ++m)
            if (t.ma[m] + t.mb[m] >= 2) out[((size_t)v * nb + m) * nc + cell] = 0.0;
        }
      }
    }
}

/* ------------------------------------------------ positivity limiter */

/* GLL nodes used by compute_set: gll = (2*(mx-1)+3)/2 points (2d/parameters_dg_2d.f90:7)
 * from gll_quadrature (2d/legendre.f90:111-170).  The reference lists -1 and 0 for its
 * two-point rule (:122-126); ref != 0 keeps that, otherwise the Lobatto nodes -1, +1. */
static int gll_nodes(int k, int ref, double *xg) {
  const int n = (2 * k + 3) / 2;
  switch (n) {
  case 2: xg[0] = -1.0; xg[1] = ref ? 0.0 : 1.0; break;
  case 3: xg[0] = -1.0; xg[1] = 0.0; xg[2] = 1.0; break;
  case 4:
    xg[0] = -1.0; xg[1] = -1.0 / 5.0 * sqrt(5.0); xg[2] = 1.0 / 5.0 * sqrt(5.0); xg[3] = 1.0;
    break;
  default: return 0;
  }
  return n;
}

/* compute_set (2d/limiters.f90:438-475): the cell polynomial at (GLL x GL) and (GL x GLL);
 * val[v][p], p = q*ng + g for the first family and nq*ng + q*ng + g for the second. */
static int positivity_set(const tabs_t *t, int ng, const double *xg, double W[NV][NBMAX],
                          double val[NV][2 * NQMAX * 4]) {
  for (int q = 0; q < t->nq; ++q)
    for (int g = 0; g < ng; ++g) {
      const int p1 = q * ng + g, p2 = t->nq * ng + q * ng + g;
      for (int v = 0; v < NV; ++v) {
        double s1 = 0.0, s2 = 0.0;
        for (int m = 0; m < t->nb; ++m) {
          s1 = s1 + W[v][m] * orc_legendre(xg[g], t->ma[m]) * orc_legendre(t->xq[q], t->mb[m]);
          s2 = s2 + W[v][m] * orc_legendre(t->xq[q], t->ma[m]) * orc_legendre(xg[g], t->mb[m]);
        }
        val[v][p1] = s1;
        val[v][p2] = s2;
      }
    }
  return 2 * t->nq * ng;
}

/* solve_for_t, 2d/limiters.f90:312-362: the root in [0,1] of p(u_avg + t (u - u_avg)) = eps,
 * written as a t^2 + b t + c = 0 with (2 rho E - |m|^2 - 2 eps rho/(gamma-1)) */
double orc_solve_for_t(const orc_cfg *c, const double *u, const double *ua) {
  const double eps = c->pos_eps, g = c->gamma;
  const double pa = ua[0], mxa = ua[1], mya = ua[2], ea = ua[3];
  const double pj = u[0], mxj = u[1], myj = u[2], ej = u[3];
  double a = 2.0 * (pj - pa) * (ej - ea) - (mxj - mxa) * (mxj - mxa) - (myj - mya) * (myj - mya);
  double b = 2.0 * (pj - pa) * (ea - eps / (g - 1)) + 2.0 * pa * (ej - ea) -
             2.0 * (mxa * (mxj - mxa) + mya * (myj - mya));
  double cc = 2.0 * pa * ea - (mxa * mxa + mya * mya) - 2.0 * eps * pa / (g - 1.0);
  b = b / a;
  cc = cc / a;
  const double D = sqrt(fabs(b * b - 4 * cc));
  const double t1 = 0.5 * (-b - D), t2 = 0.5 * (-b + D);
  double t;
  if ((t1 > -eps) && (t1 < 1.0 + eps)) t = t1;
  else if ((t2 > -eps) && (t2 < 1.0 + eps)) t = t2;
  else t = 0.0;
  t = fmin(1.0, t);
  t = fmax(0.0, t);
  return t;
}

/* compute_positivity on one cell (2d/limiters.f90:478-654): density first (theta scales the
 * non-mean density modes), then pressure on the density-limited set (t_min scales the
 * non-mean modes of every variable).  u_avg is the cell's mode (0,0). */
static void positivity_cell(const orc_cfg *c, const tabs_t *t, int ng, const double *xg,
                            double W[NV][NBMAX], double *theta_out, double *t_out) {
  const double eps = c->pos_eps;
  double val[NV][2 * NQMAX * 4], ua[NV];
  for (int v = 0; v < NV; ++v) ua[v] = W[v][0];
  int np = positivity_set(t, ng, xg, W, val);
  double pmin = val[0][0];
  for (int p = 1; p < np; ++p) pmin = fmin(pmin, val[0][p]);
  const double theta = fmin(fabs((ua[0] - eps) / (ua[0] - pmin)), 1.0);
  for (int m = 1; m < t->nb; ++m) W[0][m] = theta * W[0][m];
  np = positivity_set(t, ng, xg, W, val);
  double tmin = 1.0;
  for (int p = 0; p < np; ++p) {
    double u[NV], w[NV], tt;
    for (int v = 0; v < NV; ++v) u[v] = val[v][p];
    prim(c->gamma, u, w);
    if (w[3] > eps) tt = 1.0;
    else tt = orc_solve_for_t(c, u, ua);
    if (tmin >= tt) tmin = tt;
  }
  for (int v = 0; v < NV; ++v)
    for (int m = 1; m < t->nb; ++m) W[v][m] = tmin * W[v][m];
  if (theta_out) *theta_out = theta;
  if (t_out) *t_out = tmin;
}

void orc_ref_positivity(const orc_cfg *c, const double *in, double *out, int ref_gll,
                        double *theta_out, double *t_out) {
  tabs_t t;
  make_tabs(c, &t);
  const size_t nc = (size_t)c->nx * c->ny;
  memcpy(out, in, sizeof(double) * nc * NV * t.nb);
  double xg[4];
  const int ng = gll_nodes(c->order, ref_gll, xg);
  if (c->order < 1 || ng == 0) return;  /* mx == 1: no limiting (:519-523) */
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (size_t cell = 0; cell < nc; ++cell) {
    double W[NV][NBMAX], th, tm;
    for (int v = 0; v < NV; ++v)
      for (int m = 0; m < t.nb; ++m) W[v][m] = in[((size_t)v * t.nb + m) * nc + cell];
    positivity_cell(c, &t, ng, xg, W, &th, &tm);
    for (int v = 0; v < NV; ++v)
      for (int m = 0; m < t.nb; ++m) out[((size_t)v * t.nb + m) * nc + cell] = W[v][m];
    if (theta_out) theta_out[cell] = th;
    if (t_out) t_out[cell] = tm;
  }
}

static void eq_modes_t(const orc_cfg *c, const tabs_t *t, int i, int j, double *er, double *ee) {
  const double igm1 = 1.0 / (c->gamma - 1.0);
  for (int m = 0; m < t->nb; ++m) {
    double r = 0.0, e = 0.0;
    for (int qa = 0; qa < t->nq; ++qa)
      for (int qb = 0; qb < t->nq; ++qb) {
        double re, pe;
        orc_eq_point(c, eq_fx(c, xvol(t, i, qa)), eq_fy(c, yvol(t, j, qb)), 0, 0, &re, &pe);
        const double w = 0.25 * t->wq[qa] * t->wq[qb] * t->B[t->ma[m]][qa] * t->B[t->mb[m]][qb];
        r = r + re * w;
        e = e + pe * igm1 * w;
      }
    er[m] = r;
    ee[m] = e;
  }
}
void orc_eq_modes(const orc_cfg *c, int i, int j, double *e_rho, double *e_E) {
  tabs_t t;
  make_tabs(c, &t);
  eq_modes_t(c, &t, i, j, e_rho, e_E);
}

void orc_positivity(const orc_cfg *c, const double *in, double *out) {
  tabs_t t;
  make_tabs(c, &t);
  const int nx = c->nx;
  const size_t nc = (size_t)nx * c->ny;
  memcpy(out, in, sizeof(double) * nc * NV * t.nb);
  double xg[4];
  const int ng = gll_nodes(c->order, 0, xg);
  if (c->order < 1 || ng == 0) return;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (size_t cell = 0; cell < nc; ++cell) {
    double W[NV][NBMAX], er[NBMAX], ee[NBMAX], th, tm;
    eq_modes_t(c, &t, (int)(cell % nx), (int)(cell / nx), er, ee);
    for (int v = 0; v < NV; ++v)
      for (int m = 0; m < t.nb; ++m) {
        const double d = in[((size_t)v * t.nb + m) * nc + cell];
        W[v][m] = v == 0 ? er[m] + d : v == 3 ? ee[m] + d : d;
      }
    positivity_cell(c, &t, ng, xg, W, &th, &tm);
    if (th < 1.0 || tm < 1.0)
      for (int v = 0; v < NV; ++v)
        for (int m = 1; m < t.nb; ++m)
          out[((size_t)v * t.nb + m) * nc + cell] =
              v == 0 ? W[v][m] - er[m] : v == 3 ? W[v][m] - ee[m] : W[v][m];
  }
}

/* cell-mean equilibrium (mode (0,0) of its projection, 2d/benchmark_2d_dg.f90:530-536) */
static void eq_mean(const orc_cfg *c, const tabs_t *t, int i, int j, double *rm, double *pm) {
  double r = 0.0, p = 0.0;
  for (int qa = 0; qa < t->nq; ++qa)
    for (int qb = 0; qb < t->nq; ++qb) {
      double re, pe;
      orc_eq_point(c, eq_fx(c, xvol(t, i, qa)), eq_fy(c, yvol(t, j, qb)), 0, 0, &re, &pe);
      r = r + 0.25 * re * t->wq[qa] * t->wq[qb];
      p = p + 0.25 * pe * t->wq[qa] * t->wq[qb];
    }
  *rm = r;
  *pm = p;
}

/* Max wave speeds over cell means of the full state u_eq + delta, as
 * compute_max_speed (2d/benchmark_2d_dg.f90:826-870) intends: per direction
 * max(|v|+c), without the running-min defect of :862-864. */
void orc_max_speed(const orc_cfg *c, const double *delta, double *smax_x, double *smax_y) {
  tabs_t t;
  make_tabs(c, &t);
  const size_t nc = (size_t)c->nx * c->ny;
  const double igm1 = 1.0 / (c->gamma - 1.0);
  double sx = 0.0, sy = 0.0;
  for (int j = 0; j < c->ny; ++j)
    for (int i = 0; i < c->nx; ++i) {
      size_t cell = (size_t)j * c->nx + i;
      double rm, pm;
      eq_mean(c, &t, i, j, &rm, &pm);
      double u[NV], w[NV];
      u[0] = rm + delta[(size_t)0 * t.nb * nc + cell];
      u[1] = delta[(size_t)1 * t.nb * nc + cell];
      u[2] = delta[(size_t)2 * t.nb * nc + cell];
      u[3] = pm * igm1 + delta[(size_t)3 * t.nb * nc + cell];
      prim(c->gamma, u, w);
      double cs = sound(c->gamma, w);
      sx = fmax(sx, fabs(w[1]) + cs);
      sy = fmax(sy, fabs(w[2]) + cs);
    }
  *smax_x = sx;
  *smax_y = sy;
}

/* CFL time step for degree k: cfl / ((2k+1) (sx/dx + sy/dy)); the (2k+1) factor of
 * dg_with_source.f90:178 with directional speeds in place of :671's mixed values. */
double orc_cfl_dt(const orc_cfg *c, double smax_x, double smax_y) {
  double dx = c->lx / (double)c->nx, dy = c->ly / (double)c->ny;
  return c->cfl / ((2.0 * c->order + 1.0) * (smax_x / dx + smax_y / dy));
}

/* SSP-RK2 'EQL' branch of evolve, 2d/benchmark_2d_dg.f90:672-681 (limiter after
 * each stage, and once before the loop, :657) */
double orc_run_rk2(const orc_cfg *c, double *delta, int nsteps, double dt_fixed) {
  const size_t n = (size_t)c->nx * c->ny * NV * orc_nb(c->order, c->basis);
  double *L = (double *)malloc(n * sizeof(double)), *w1 = (double *)malloc(n * sizeof(double));
  double *tmp = (double *)malloc(n * sizeof(double));
  double t = 0.0;
  orc_limit(c, delta, tmp);
  memcpy(delta, tmp, n * sizeof(double));
  for (int it = 0; it < nsteps; ++it) {
    double dt = dt_fixed;
    if (!(dt_fixed > 0.0)) {
      double sx, sy;
      orc_max_speed(c, delta, &sx, &sy);
      dt = orc_cfl_dt(c, sx, sy);
    }
    orc_rhs(c, delta, L);
    for (size_t e = 0; e < n; ++e) tmp[e] = delta[e] + dt * L[e];
    orc_limit(c, tmp, w1);
    orc_rhs(c, w1, L);
    for (size_t e = 0; e < n; ++e) tmp[e] = 0.5 * delta[e] + 0.5 * w1[e] + 0.5 * dt * L[e];
    orc_limit(c, tmp, delta);
    t += dt;
  }
  free(L);
  free(w1);
  free(tmp);
  return t;
}

/* SSP-RK(5,4) 'RK4' branch of evolve, 2d/benchmark_2d_dg.f90:683-710 (its repeated
 * compute_update(w3) at :700 recomputes the L(w3) already held) */
double orc_run_rk54(const orc_cfg *c, double *delta, int nsteps, double dt_fixed) {
  const size_t n = (size_t)c->nx * c->ny * NV * orc_nb(c->order, c->basis);
  double *L = malloc(n * 8), *L3 = malloc(n * 8), *w1 = malloc(n * 8), *w2 = malloc(n * 8);
  double *w3 = malloc(n * 8), *w4 = malloc(n * 8), *tmp = malloc(n * 8);
  double t = 0.0;
  orc_limit(c, delta, tmp);
  memcpy(delta, tmp, n * 8);
  for (int it = 0; it < nsteps; ++it) {
    double dt = dt_fixed;
    if (!(dt_fixed > 0.0)) {
      double sx, sy;
      orc_max_speed(c, delta, &sx, &sy);
      dt = orc_cfl_dt(c, sx, sy);
    }
    orc_rhs(c, delta, L);
    for (size_t e = 0; e < n; ++e) tmp[e] = delta[e] + 0.391752226571890 * dt * L[e];
    orc_limit(c, tmp, w1);
    orc_rhs(c, w1, L);
    for (size_t e = 0; e < n; ++e)
      tmp[e] = 0.444370493651235 * delta[e] + 0.555629506348765 * w1[e] +
               0.368410593050371 * dt * L[e];
    orc_limit(c, tmp, w2);
    orc_rhs(c, w2, L);
    for (size_t e = 0; e < n; ++e)
      tmp[e] = 0.620101851488403 * delta[e] + 0.379898148511597 * w2[e] +
               0.251891774271694 * dt * L[e];
    orc_limit(c, tmp, w3);
    orc_rhs(c, w3, L3);
    for (size_t e = 0; e < n; ++e)
      tmp[e] = 0.178079954393132 * delta[e] + 0.821920045606868 * w3[e] +
               0.544974750228521 * dt * L3[e];
    orc_limit(c, tmp, w4);
    orc_rhs(c, w4, L);
    for (size_t e = 0; e < n; ++e)
      tmp[e] = 0.00683325884039 * delta[e] + 0.51723167208978 * w2[e] + 0.12759831133288 * w3[e] +
               0.34833675773694 * w4[e] + 0.08460416338212 * dt * L3[e] +
               0.22600748319395 * dt * L[e];
    orc_limit(c, tmp, delta);
    t += dt;
  }
  free(L); free(L3); free(w1); free(w2); free(w3); free(w4); free(tmp);
  return t;
}

/* compute_error norms, 2d/benchmark_2d_dg.f90:23-89, of a - b (nodal values at the
 * GL points, weights w_x*w_y, area dx*dy/4); l2 returned as its square root */
void orc_norms(const orc_cfg *c, const double *a, const double *b, double *l1, double *linf,
               double *l2) {
  tabs_t t;
  make_tabs(c, &t);
  const size_t nc = (size_t)c->nx * c->ny;
  const int nq2 = t.nq * t.nq;
  double *na = malloc(sizeof(double) * nc * NV * nq2), *nb_ = malloc(sizeof(double) * nc * NV * nq2);
  orc_nodes_from_modes(c, NV, a, na);
  orc_nodes_from_modes(c, NV, b, nb_);
  for (int v = 0; v < NV; ++v) {
    double s1 = 0.0, s2 = 0.0, mx = 0.0;
    for (size_t cell = 0; cell < nc; ++cell) {
      double acc1 = 0.0, acc2 = 0.0;
      for (int qa = 0; qa < t.nq; ++qa)
        for (int qb = 0; qb < t.nq; ++qb) {
          size_t e = ((size_t)v * nq2 + qa * t.nq + qb) * nc + cell;
          double d = na[e] - nb_[e];
          acc1 = acc1 + fabs(d) * t.wq[qa] * t.wq[qb];
          acc2 = acc2 + d * d * t.wq[qa] * t.wq[qb];
          mx = fmax(mx, fabs(d));
        }
      s1 = s1 + acc1 * (t.dx * t.dy) * 0.25;
      s2 = s2 + acc2 * (t.dx * t.dy) * 0.25;
    }
    l1[v] = s1;
    l2[v] = sqrt(s2);
    linf[v] = mx;
  }
  free(na);
  free(nb_);
}

/* ------------------------- literal restatement of the reference 2D DG operator */

/*
 * compute_update, 2d/benchmark_2d_dg.f90:1137-1479, plain (nequilibrium=3) form, with
 * the Fortran layout u(nvar,nx,ny,mx,my).  bc: 1 periodic, 2 copy
 * (get_boundary_conditions :777-824; the x faces use dim=2 as at :1338-1339).
 */
#define FIDX(v, i, j, a, b) ((v) + NV * ((size_t)(i) + (size_t)nx * ((j) + (size_t)ny * ((a) + (size_t)m * (b)))))
static int ref_bc(int index, int n, int bc) {
  if (bc == 1) {
    if (index == 0) return n;
    if (index == n + 1) return 1;
  } else if (bc == 2 || bc == 3) {
    if (index == 0) return 1;
    if (index == n + 1) return n;
  }
  return index;
}
void orc_ref2d_compute_update(int nx, int ny, int m, double gamma, double lx, double ly,
                              int ref_flux_bug, int ref_source, int grad_phi_bug, double gx,
                              double gy, int bc, const double *u, double *dudt) {
  (void)ly;
  double xq[NQMAX], wq[NQMAX];
  orc_gl_quadrature(m, xq, wq);
  const double dx = lx / (double)nx, dy = ly / (double)ny;
  const double oneoverdx = 1. / dx;
  const size_t ntot = (size_t)NV * nx * ny * m * m;
  double *nodes = calloc(ntot, 8), *f1 = calloc(ntot, 8), *f2 = calloc(ntot, 8);
  double *vol1 = calloc(ntot, 8), *vol2 = calloc(ntot, 8), *src = calloc(ntot, 8);
  /* traces: [v][i][j][q] */
  size_t ntr = (size_t)NV * nx * ny * m;
  double *uL = calloc(ntr, 8), *uR = calloc(ntr, 8), *uT = calloc(ntr, 8), *uB = calloc(ntr, 8);
  /* F(v, q, iface 1..nx+1, j), G(v, q, i, jface 1..ny+1) */
  double *F = calloc((size_t)NV * m * (nx + 1) * ny, 8), *G = calloc((size_t)NV * m * nx * (ny + 1), 8);
#define TR(v, i, j, q) ((v) + NV * ((size_t)(i) + (size_t)nx * ((j) + (size_t)ny * (q))))
#define FF(v, q, f, j) ((v) + NV * ((q) + (size_t)m * ((f) + (size_t)(nx + 1) * (j))))
#define GG(v, q, i, f) ((v) + NV * ((q) + (size_t)m * ((i) + (size_t)nx * (f))))
  /* get_nodes_from_modes :544-592 */
  for (int v = 0; v < NV; ++v)
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int a = 0; a < m; ++a)
          for (int b = 0; b < m; ++b) {
            double s = 0.0;
            for (int p = 0; p < m; ++p)
              for (int q = 0; q < m; ++q)
                s = s + u[FIDX(v, i, j, p, q)] * orc_legendre(xq[a], p) * orc_legendre(xq[b], q);
            nodes[FIDX(v, i, j, a, b)] = s;
          }
  /* compute_flux :919-942 */
  for (size_t p = 0; p < ntot / NV; ++p) {
    const double *un = nodes + NV * p;
    double w[NV];
    prim(gamma, un, w);
    double *a1 = f1 + NV * p, *a2 = f2 + NV * p;
    a2[0] = w[0] * w[2];
    a2[1] = w[0] * w[1] * w[2];
    a2[2] = w[2] * un[2] + w[3];
    a2[3] = w[2] * un[3] + w[2] * w[3];
    a1[0] = w[0] * w[1];
    a1[1] = w[1] * un[1] + w[3];
    a1[2] = w[0] * w[1] * w[2];
    a1[3] = w[1] * un[3] + w[1] * w[3];
  }
  /* volume integrals :1207-1244 */
  for (int v = 0; v < NV; ++v)
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int a = 0; a < m; ++a)
          for (int b = 0; b < m; ++b) {
            double s1 = 0.0, s2 = 0.0;
            for (int p = 0; p < m; ++p)
              for (int q = 0; q < m; ++q)
                s1 = s1 + f1[FIDX(v, i, j, p, q)] * orc_legendre_prime(xq[p], a) * wq[p] *
                              orc_legendre(xq[q], b) * wq[q];
            for (int p = 0; p < m; ++p)
              for (int q = 0; q < m; ++q)
                s2 = s2 + f2[FIDX(v, i, j, p, q)] * orc_legendre_prime(xq[q], b) * wq[q] *
                              orc_legendre(xq[p], a) * wq[p];
            vol1[FIDX(v, i, j, a, b)] = s1;
            vol2[FIDX(v, i, j, a, b)] = s2;
          }
  /* traces :1253-1314 */
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int v = 0; v < NV; ++v)
        for (int q = 0; q < m; ++q) {
          double l = 0, r = 0, bt = 0, tp = 0;
          for (int a = 0; a < m; ++a)
            for (int b = 0; b < m; ++b) {
              double d = u[FIDX(v, i, j, a, b)];
              l = l + d * orc_legendre(-1.0, a) * orc_legendre(xq[q], b);
              r = r + d * orc_legendre(1.0, a) * orc_legendre(xq[q], b);
              bt = bt + d * orc_legendre(-1.0, b) * orc_legendre(xq[q], a);
              tp = tp + d * orc_legendre(1.0, b) * orc_legendre(xq[q], a);
            }
          uL[TR(v, i, j, q)] = l;
          uR[TR(v, i, j, q)] = r;
          uB[TR(v, i, j, q)] = bt;
          uT[TR(v, i, j, q)] = tp;
        }
  /* faces :1333-1366 with compute_num_flux :991-1006 -> compute_llflux :968-988 */
  orc_cfg cc;
  memset(&cc, 0, sizeof(cc));
  cc.gamma = gamma;
  cc.llf_speed = ORC_LLF_REF2D;
  if (!ref_flux_bug) {
    for (int j = 1; j <= ny; ++j)
      for (int f = 1; f <= nx + 1; ++f) {
        int il = ref_bc(f - 1, ny, bc), ir = ref_bc(f, ny, bc);
        for (int q = 0; q < m; ++q) {
          double a[NV], b[NV], fh[NV];
          for (int v = 0; v < NV; ++v) {
            a[v] = uR[TR(v, il - 1, j - 1, q)];
            b[v] = uL[TR(v, ir - 1, j - 1, q)];
          }
          llf(&cc, a, b, 0, fh);
          for (int v = 0; v < NV; ++v) F[FF(v, q, f - 1, j - 1)] = fh[v];
        }
      }
    for (int i = 1; i <= nx; ++i)
      for (int f = 1; f <= ny + 1; ++f) {
        int jl = ref_bc(f - 1, ny, bc), jr = ref_bc(f, ny, bc);
        for (int q = 0; q < m; ++q) {
          double a[NV], b[NV], fh[NV];
          for (int v = 0; v < NV; ++v) {
            a[v] = uT[TR(v, i - 1, jl - 1, q)];
            b[v] = uB[TR(v, i - 1, jr - 1, q)];
          }
          llf(&cc, a, b, 1, fh);
          for (int v = 0; v < NV; ++v) G[GG(v, q, i - 1, f - 1)] = fh[v];
        }
      }
  }
  /* source :1415-1443 (get_source :1558-1576, grad_phi :1599-1644) */
  if (ref_source == 2) {
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j) {
        double sq[NQMAX][NQMAX][NV];
        for (int p = 0; p < m; ++p)
          for (int q = 0; q < m; ++q) {
            double w[NV], gpx, gpy;
            prim(gamma, nodes + FIDX(0, i, j, p, q), w);
            if (grad_phi_bug) {
              gpx = ((double)(float)(i + 0.5f)) * dx + dx / 2.0 * xq[p];
              gpy = ((double)(float)(j + 0.5f)) * dy + dy / 2.0 * xq[q];
              sq[p][q][0] = 0.;
              sq[p][q][1] = w[0] * gpx;
              sq[p][q][2] = w[0] * gpy;
              sq[p][q][3] = w[0] * (w[1] * gpx + w[2] * gpy);
            } else {
              source(w, gx, gy, sq[p][q]);
            }
          }
        for (int v = 0; v < NV; ++v)
          for (int a = 0; a < m; ++a)
            for (int b = 0; b < m; ++b) {
              double s = 0.0;
              for (int p = 0; p < m; ++p)
                for (int q = 0; q < m; ++q)
                  s = s + sq[p][q][v] * orc_legendre(xq[p], a) * wq[p] * orc_legendre(xq[q], b) * wq[q];
              src[FIDX(v, i, j, a, b)] = s;
            }
      }
  }
  /* edge integrals :1372-1411 and assembly :1449-1466 */
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int v = 0; v < NV; ++v)
        for (int a = 0; a < m; ++a)
          for (int b = 0; b < m; ++b) {
            double e1 = 0, e2 = 0, e3 = 0, e4 = 0;
            for (int q = 0; q < m; ++q) {
              e1 = e1 + F[FF(v, q, i + 1, j)] * orc_legendre(1.0, a) * orc_legendre(xq[q], b) * wq[q];
              e2 = e2 + F[FF(v, q, i, j)] * orc_legendre(-1.0, a) * orc_legendre(xq[q], b) * wq[q];
            }
            for (int q = 0; q < m; ++q) {
              e3 = e3 + G[GG(v, q, i, j + 1)] * orc_legendre(1.0, b) * orc_legendre(xq[q], a) * wq[q];
              e4 = e4 + G[GG(v, q, i, j)] * orc_legendre(-1.0, b) * orc_legendre(xq[q], a) * wq[q];
            }
            size_t e = FIDX(v, i, j, a, b);
            dudt[e] = (oneoverdx * vol1[e] + oneoverdx * vol2[e] - oneoverdx * (e1 - e2) -
                       oneoverdx * (e3 - e4)) / 2. + src[e] / 4.;
          }
  free(nodes); free(f1); free(f2); free(vol1); free(vol2); free(src);
  free(uL); free(uR); free(uT); free(uB); free(F); free(G);
#undef TR
#undef FF
#undef GG
}
#undef FIDX

/* ------------------------------- literal restatement of the 1D WB DG operator */

/* 1D physics of dg_with_source.f90:1167-1316 (nvar = 3) */
static inline void prim1(double g, const double *u, double *w) {
  w[0] = u[0];
  w[1] = u[1] / w[0];
  w[2] = (g - 1.0) * (u[2] - 0.5 * w[0] * (w[1] * w[1]));
}
static inline void flux1(double g, const double *u, double *f) {
  double w[3];
  prim1(g, u, w);
  f[0] = w[1] * u[0];
  f[1] = w[1] * u[1] + w[2];
  f[2] = w[1] * u[2] + w[2] * w[1];
}
static inline double speed1(double g, const double *u) {
  double w[3];
  prim1(g, u, w);
  return fabs(w[1]) + sqrt(g * fmax(w[2], 1e-10) / fmax(w[0], 1e-10));
}
static inline void llf1(double g, const double *ul, const double *ur, double *f) {
  double fl[3], fr[3];
  double cmax = fmax(speed1(g, ul), speed1(g, ur));
  flux1(g, ul, fl);
  flux1(g, ur, fr);
  for (int v = 0; v < 3; ++v) f[v] = 0.5 * (fr[v] + fl[v]) - 0.5 * cmax * (ur[v] - ul[v]);
}
/* riemann_hllc, dg_with_source.f90:1318-1374: acoustic star state from the Lagrangian
 * sound speeds, sampled at x/t = 0, flux of the sampled state */
void orc_ref_riemann_hllc(double g, const double *ul, const double *ur, double *fg) {
  double wl[3], wr[3], wst[3], wstl[3], wstr[3], ustl[3], ustr[3], wgd[3], ugd[3];
  prim1(g, ul, wl);
  prim1(g, ur, wr);
  const double cl = sqrt(g * fmax(wl[2], 1e-10) / fmax(wl[0], 1e-10));
  const double cr = sqrt(g * fmax(wr[2], 1e-10) / fmax(wr[0], 1e-10));
  const double SL = fmin(wl[1], wr[1]) - fmax(cl, cr);
  const double SR = fmax(wl[1], wr[1]) + fmax(cl, cr);
  const double DL = wl[0] * (wl[1] - SL);
  const double DR = wr[0] * (SR - wr[1]);
  wst[1] = (DR * wr[1] + DL * wl[1] + (wl[2] - wr[2])) / (DL + DR);
  wst[2] = (DR * wl[2] + DL * wr[2] + DL * DR * (wl[1] - wr[1])) / (DL + DR);
  wstl[0] = wl[0] * (SL - wl[1]) / (SL - wst[1]);
  ustl[2] = ((SL - wl[1]) * ul[2] - wl[2] * wl[1] + wst[2] * wst[1]) / (SL - wst[1]);
  wstr[0] = wr[0] * (SR - wr[1]) / (SR - wst[1]);
  ustr[2] = ((SR - wr[1]) * ur[2] - wr[2] * wr[1] + wst[2] * wst[1]) / (SR - wst[1]);
  if (SL > 0.0) {
    wgd[0] = wl[0]; wgd[1] = wl[1]; wgd[2] = wl[2]; ugd[2] = ul[2];
  } else if (wst[1] > 0.0) {
    wgd[0] = wstl[0]; wgd[1] = wst[1]; wgd[2] = wst[2]; ugd[2] = ustl[2];
  } else if (SR > 0.0) {
    wgd[0] = wstr[0]; wgd[1] = wst[1]; wgd[2] = wst[2]; ugd[2] = ustr[2];
  } else {
    wgd[0] = wr[0]; wgd[1] = wr[1]; wgd[2] = wr[2]; ugd[2] = ur[2];
  }
  fg[0] = wgd[0] * wgd[1];
  fg[1] = wgd[0] * wgd[1] * wgd[1] + wgd[2];
  fg[2] = wgd[1] * (ugd[2] + wgd[2]);
}

static inline void source1(double g, const double *u, double *s) {
  double w[3];
  prim1(g, u, w);
  s[0] = 0;
  s[1] = -w[0];
  s[2] = -w[0] * w[1];
}

/*
 * compute_update_exact_delta, dg_with_source.f90:1749-2031, with riemann_llf
 * (riemann=1) or riemann_hllc (riemann=2, :1909-1917), equilibrium rho = p = exp(-x) (get_eq_solution :1031-1048) and the
 * sqrt(2n+1) basis of 2d/legendre.f90 (for which the 1/dx and 0.5 factors of
 * :1998-2025 are the consistent ones).  Out-of-range faces wrap periodically; the
 * two end cells are frozen (:2028-2029) so they never reach the result.
 */
void orc_dg1d_update_exact_delta(int nx, int n, double g, double lx, int half_source,
                                 int riemann, const double *du, double *dudt) {
#define D1(v, i, c) ((v) + 3 * ((i) + (size_t)n * (c)))
  double xq[NQMAX], wq[NQMAX];
  orc_gl_quadrature(n, xq, wq);
  const double dx = lx / (double)nx, oneoverdx = 1. / dx;
  const double igm1 = 1.0 / (g - 1.0);
  double *fv = calloc((size_t)3 * n * nx, 8), *fve = calloc((size_t)3 * n * nx, 8);
  double *sv = calloc((size_t)3 * n * nx, 8), *sve = calloc((size_t)3 * n * nx, 8);
  double *uface = calloc((size_t)3 * (nx + 1), 8), *fface = calloc((size_t)3 * (nx + 1), 8);
  double *fface_eq = calloc((size_t)3 * (nx + 1), 8);
  double *ul = calloc((size_t)3 * nx, 8), *ur = calloc((size_t)3 * nx, 8);
  for (int f = 0; f <= nx; ++f) {
    double x = (double)f * dx, e = exp(-x);
    uface[3 * f + 0] = e;
    uface[3 * f + 1] = e * 0.0;
    uface[3 * f + 2] = e / (g - 1.0) + 0.5 * e * 0.0;
    flux1(g, uface + 3 * f, fface_eq + 3 * f);
  }
  for (int c = 0; c < nx; ++c) {
    double xc = ((double)c + 0.5) * dx;
    double fq[NQMAX][3], fqe[NQMAX][3], sq[NQMAX][3], sqe[NQMAX][3];
    for (int j = 0; j < n; ++j) {
      double xj = xc + dx / 2.0 * xq[j], e = exp(-xj);
      double ue[3] = {e, e * 0.0, e / (g - 1.0) + 0.5 * e * 0.0}, uq[3] = {0, 0, 0}, ut[3];
      for (int v = 0; v < 3; ++v)
        for (int i = 0; i < n; ++i) uq[v] = uq[v] + du[D1(v, i, c)] * orc_legendre(xq[j], i);
      for (int v = 0; v < 3; ++v) ut[v] = ue[v] + uq[v];
      flux1(g, ut, fq[j]);
      flux1(g, ue, fqe[j]);
      source1(g, ut, sq[j]);
      source1(g, ue, sqe[j]);
    }
    for (int v = 0; v < 3; ++v)
      for (int i = 0; i < n; ++i) {
        double a = 0, b = 0, s = 0, se = 0;
        for (int j = 0; j < n; ++j) {
          a = a + fq[j][v] * orc_legendre_prime(xq[j], i) * wq[j];
          b = b + fqe[j][v] * orc_legendre_prime(xq[j], i) * wq[j];
          double h = half_source ? 0.5 : 1.0;
          s = s + sq[j][v] * orc_legendre(xq[j], i) * wq[j] * h;
          se = se + sqe[j][v] * orc_legendre(xq[j], i) * wq[j] * h;
        }
        fv[D1(v, i, c)] = a;
        fve[D1(v, i, c)] = b;
        sv[D1(v, i, c)] = s;
        sve[D1(v, i, c)] = se;
      }
    for (int v = 0; v < 3; ++v) {
      double l = 0, r = 0;
      for (int i = 0; i < n; ++i) {
        l = l + du[D1(v, i, c)] * orc_legendre(-1.0, i);
        r = r + du[D1(v, i, c)] * orc_legendre(1.0, i);
      }
      ul[3 * c + v] = uface[3 * c + v] + l;
      ur[3 * c + v] = uface[3 * (c + 1) + v] + r;
    }
    (void)igm1;
  }
  for (int f = 0; f <= nx; ++f) {
    int il = f - 1 < 0 ? nx - 1 : f - 1, ir = f > nx - 1 ? 0 : f;
    if (riemann == 2) orc_ref_riemann_hllc(g, ur + 3 * il, ul + 3 * ir, fface + 3 * f);
    else llf1(g, ur + 3 * il, ul + 3 * ir, fface + 3 * f);
  }
  for (int c = 0; c < nx; ++c)
    for (int i = 0; i < n; ++i)
      for (int v = 0; v < 3; ++v) {
        double pr = orc_legendre(1.0, i), pl = orc_legendre(-1.0, i);
        dudt[D1(v, i, c)] =
            oneoverdx * fv[D1(v, i, c)] - oneoverdx * fve[D1(v, i, c)] -
            oneoverdx * (fface[3 * (c + 1) + v] * pr - fface[3 * c + v] * pl) +
            oneoverdx * (fface_eq[3 * (c + 1) + v] * pr - fface_eq[3 * c + v] * pl) +
            sv[D1(v, i, c)] - sve[D1(v, i, c)];
        if (c == 0 || c == nx - 1) dudt[D1(v, i, c)] = 0.0;
      }
  free(fv); free(fve); free(sv); free(sve); free(uface); free(fface); free(fface_eq);
  free(ul); free(ur);
#undef D1
}

/* ----------------------------------------------- 1D well-balanced FV (config 1) */

static void fv1d_eq(const orc_fv1d_cfg *c, double x, double *r, double *p) {
  orc_cfg cc;
  memset(&cc, 0, sizeof(cc));
  cc.eq_kind = c->eq_kind;
  cc.gamma = c->gamma;
  cc.gx = c->g;
  cc.gy = 0.0;
  cc.rho0 = c->rho0;
  cc.p0 = c->p0;
  cc.kpoly = c->kpoly;
  orc_eq_at(&cc, x, 0.0, r, p);
}
void orc_fv1d_eq_cells(const orc_fv1d_cfg *c, double *rho, double *p) {
  double dx = c->lx / (double)c->nx;
  for (int i = 0; i < c->nx; ++i) fv1d_eq(c, ((double)i + 0.5) * dx, rho + i, p + i);
}

/* 1D primitive/flux/speed of benchmark_1d.f90:112-198 */
static inline void fv_prim(double g, const double *u, double *w) {
  w[0] = u[0];
  w[1] = u[1] / w[0];
  w[2] = (g - 1.0) * (u[2] - 0.5 * w[0] * w[1] * w[1]);
}
static inline void fv_flux(double g, const double *u, double *f) {
  double w[3];
  fv_prim(g, u, w);
  f[0] = w[1] * u[0];
  f[1] = w[1] * u[1] + w[2];
  f[2] = w[1] * u[2] + w[2] * w[1];
}
static inline double fv_speed(double g, const double *u) {
  double w[3];
  fv_prim(g, u, w);
  return fabs(w[1]) + sqrt(g * fmax(w[2], 1e-10) / fmax(w[0], 1e-10));
}

/*
 * Well-balanced FV update, compute_update 'EQL' (benchmark_1d.f90:263-377):
 * face states u_eq(x_face) + delta (:296-303), LLF (:438-451), equilibrium face flux
 * subtracted (:371-372), source -rho g, -m g (get_source :379-405 with the centred
 * (x+ - x-)/(2 dx) = 1 factor of a linear potential).  Second order by minmod MUSCL
 * on delta (minmod, limiters.f90:1-21); bc 1 copies delta into the ghost cells
 * (u_eq(ghost) + delta(edge)).  Differences are formed per face and per cell so a
 * zero perturbation gives an exactly zero update.
 */
/*
 * 'WB1' update, compute_update_sr (benchmark_1d.f90:553-747), on the full state
 * u_i = u_eq(x_i) + delta_i: per cell the specific enthalpy h = p/rho (1 + 1/(gamma-1))
 * and K = p / rho^gamma, both with the default-real floor 1e-5 (:611,619); h moved to the
 * faces along h + Phi = const (:615-616, Phi = g x); face states of the cell's own K
 * with the cell velocity (:631-635); LLF of the adjacent face states on the interior
 * faces (:642-666, compute_llflux :438-451); source (0, (p_right - p_left)/dx,
 * -rho v g (x+ - x-)/(2 dx)) (get_source_rg :409-434); the two end cells take their
 * neighbour's update (:741-742).  The reference's 1/dx is boxlen/dx and its source
 * spacing 1/nx, which agree with dx for its boxlen = 1; dx is used here.
 */
static void wb1_face_states(const orc_fv1d_cfg *c, const double *d, const double *re,
                            const double *pe, int i, double dx, double *uL, double *uR,
                            double *pL, double *pR, double *w) {
  const double g = c->gamma, fl = (double)1e-5f;
  double u[3] = {re[i] + d[3 * i], d[3 * i + 1], pe[i] / (g - 1.0) + d[3 * i + 2]};
  fv_prim(g, u, w);
  const double h = fmax(w[2], fl) / fmax(fl, w[0]) * (1 + 1. / (g - 1));
  const double xc = ((double)i + 0.5) * dx, xl = (double)i * dx, xr = (double)(i + 1) * dx;
  const double h0l = h + c->g * xc - c->g * xl, h0r = h + c->g * xc - c->g * xr;
  const double K = fmax(fl, w[2]) / pow(fmax(fl, w[0]), g);
  const double rl = pow((1. / K) * (g - 1) / g * h0l, 1 / (g - 1));
  const double rr = pow((1. / K) * (g - 1) / g * h0r, 1 / (g - 1));
  *pL = pow(1. / K, 1 / (g - 1)) * pow((g - 1) / g * h0l, g / (g - 1));
  *pR = pow(1. / K, 1 / (g - 1)) * pow((g - 1) / g * h0r, g / (g - 1));
  uL[0] = rl;
  uL[1] = rl * w[1];
  uL[2] = *pL / (g - 1.0) + 0.5 * rl * w[1] * w[1];
  uR[0] = rr;
  uR[1] = rr * w[1];
  uR[2] = *pR / (g - 1.0) + 0.5 * rr * w[1] * w[1];
}

static void wb1_rhs(const orc_fv1d_cfg *c, const double *d, double *dudt) {
  const int nx = c->nx;
  const double dx = c->lx / (double)nx, g = c->gamma;
  double *re = malloc(sizeof(double) * nx), *pe = malloc(sizeof(double) * nx);
  double *fh = calloc((size_t)3 * (nx + 1), 8);
  orc_fv1d_eq_cells(c, re, pe);
  for (int f = 1; f < nx; ++f) {
    double aL[3], aR[3], bL[3], bR[3], p1, p2, p3, p4, w[3], fa[3], fb[3];
    wb1_face_states(c, d, re, pe, f - 1, dx, aL, aR, &p1, &p2, w);  /* cell left of f */
    wb1_face_states(c, d, re, pe, f, dx, bL, bR, &p3, &p4, w);      /* cell right of f */
    fv_flux(g, aR, fa);
    fv_flux(g, bL, fb);
    const double cmax = fmax(fv_speed(g, aR), fv_speed(g, bL));
    for (int v = 0; v < 3; ++v) fh[3 * f + v] = 0.5 * (fb[v] + fa[v]) - 0.5 * cmax * (bL[v] - aR[v]);
  }
  for (int i = 1; i < nx - 1; ++i) {
    double uL[3], uR[3], pL, pR, w[3];
    wb1_face_states(c, d, re, pe, i, dx, uL, uR, &pL, &pR, w);
    const double xm = ((double)(i - 1) + 0.5) * dx, xp = ((double)(i + 1) + 0.5) * dx;
    const double s[3] = {0.0, (pR - pL) / dx, -w[0] * w[1] * c->g * (xp - xm) / (2 * dx)};
    for (int v = 0; v < 3; ++v)
      dudt[3 * i + v] = -(fh[3 * (i + 1) + v] - fh[3 * i + v]) / dx + s[v];
  }
  for (int v = 0; v < 3; ++v) {
    dudt[v] = dudt[3 + v];
    dudt[3 * (nx - 1) + v] = dudt[3 * (nx - 2) + v];
  }
  free(re);
  free(pe);
  free(fh);
}

void orc_fv1d_rhs(const orc_fv1d_cfg *c, const double *d, double *dudt) {
  if (c->scheme == 1) {
    wb1_rhs(c, d, dudt);
    return;
  }
  const int nx = c->nx;
  const double dx = c->lx / (double)nx, g = c->gamma, igm1 = 1.0 / (c->gamma - 1.0);
  double *sl = calloc((size_t)3 * (nx + 2), 8); /* slopes incl. ghosts at 0 and nx+1 */
  double *dg = calloc((size_t)3 * (nx + 4), 8); /* delta with 2 ghosts each side */
  double *fh = calloc((size_t)3 * (nx + 1), 8);
  for (int i = -2; i < nx + 2; ++i) {
    int s;
    if (c->bc == 0) s = ((i % nx) + nx) % nx;
    else s = i < 0 ? 0 : (i >= nx ? nx - 1 : i);
    for (int v = 0; v < 3; ++v) dg[3 * (i + 2) + v] = d[3 * s + v];
  }
  for (int i = -1; i <= nx; ++i)
    for (int v = 0; v < 3; ++v) {
      double sg = 0.0;
      if (c->limiter) {
        double dp = dg[3 * (i + 3) + v] - dg[3 * (i + 2) + v];
        double dm = dg[3 * (i + 2) + v] - dg[3 * (i + 1) + v];
        sg = minmod3(dp, dm, dm);
      }
      if (c->bc != 0 && (i < 0 || i >= nx)) sg = 0.0;
      sl[3 * (i + 1) + v] = sg;
    }
  for (int f = 0; f <= nx; ++f) {
    double re, pe;
    fv1d_eq(c, (double)f * dx, &re, &pe);
    double ue[3] = {re, 0.0, pe * igm1}, uL[3], uR[3], fl[3], fr[3], fe[3];
    for (int v = 0; v < 3; ++v) {
      uL[v] = ue[v] + (dg[3 * (f + 1) + v] + 0.5 * sl[3 * f + v]);
      uR[v] = ue[v] + (dg[3 * (f + 2) + v] - 0.5 * sl[3 * (f + 1) + v]);
    }
    fv_flux(g, uL, fl);
    fv_flux(g, uR, fr);
    fv_flux(g, ue, fe);
    double cmax = fmax(fv_speed(g, uL), fv_speed(g, uR));
    for (int v = 0; v < 3; ++v)
      fh[3 * f + v] = (0.5 * (fr[v] + fl[v]) - 0.5 * cmax * (uR[v] - uL[v])) - fe[v];
  }
  for (int i = 0; i < nx; ++i) {
    double re, pe;
    fv1d_eq(c, ((double)i + 0.5) * dx, &re, &pe);
    double r = re + d[3 * i + 0];
    double s1 = -(r * c->g) - (-(re * c->g));
    double s2 = -(d[3 * i + 1] * c->g);
    double s[3] = {0.0, s1, s2};
    for (int v = 0; v < 3; ++v)
      dudt[3 * i + v] = -(fh[3 * (i + 1) + v] - fh[3 * i + v]) / dx + s[v];
  }
  free(sl);
  free(dg);
  free(fh);
}

/* evolve 'EQL' with a genuine SSP-RK2 second stage (benchmark_1d.f90:200-261 evaluates
 * it on u, a forward-Euler defect) and dt = cfl dx / max(|u|+c), clipped at tend */
double orc_fv1d_run(const orc_fv1d_cfg *c, double *d, double tend, int max_steps,
                    int *steps_done) {
  const int nx = c->nx;
  const double dx = c->lx / (double)nx, igm1 = 1.0 / (c->gamma - 1.0);
  double *L = malloc(sizeof(double) * 3 * nx), *w1 = malloc(sizeof(double) * 3 * nx);
  double *re = malloc(sizeof(double) * nx), *pe = malloc(sizeof(double) * nx);
  orc_fv1d_eq_cells(c, re, pe);
  double t = 0.0;
  int it = 0;
  while (t < tend && it < max_steps) {
    double cmax = 0.0;
    for (int i = 0; i < nx; ++i) {
      double u[3] = {re[i] + d[3 * i], d[3 * i + 1], pe[i] * igm1 + d[3 * i + 2]};
      cmax = fmax(cmax, fv_speed(c->gamma, u));
    }
    double dt = c->cfl * dx / cmax;
    if (dt > tend - t) dt = tend - t;
    orc_fv1d_rhs(c, d, L);
    for (int e = 0; e < 3 * nx; ++e) w1[e] = d[e] + dt * L[e];
    orc_fv1d_rhs(c, w1, L);
    for (int e = 0; e < 3 * nx; ++e) d[e] = 0.5 * d[e] + 0.5 * w1[e] + 0.5 * dt * L[e];
    t += dt;
    ++it;
  }
  if (steps_done) *steps_done = it;
  free(L);
  free(w1);
  free(re);
  free(pe);
  return t;
}
