/*
 * wb_oracle.h -- CPU restatement of the reference's well-balanced Euler-with-gravity
 * step (hanveiga/fvm-source-wb), used ONLY as test infrastructure: the parity checker
 * for the CUDA path and the timed CPU baseline.  Nothing in the product library links
 * or calls this code.
 *
 * Parity status: the reference is Fortran 90 and no Fortran compiler exists in the
 * build image, so the reference cannot be run here.  The basis/quadrature part is
 * pinned by known-answer tests (closed-form Legendre values, closed-form Gauss-Legendre
 * nodes/weights, and the modes<->nodes round trip of 2d/test2d.f90:77-84).  The
 * operator itself has no golden vectors in the reference: PARITY UNPINNED for the
 * operator beyond those KATs and beyond the cross-checks against the literal
 * restatements below (orc_ref2d_compute_update, orc_dg1d_update_exact_delta).
 *
 * Layout: modal state is SoA, u[(v*nb + m)*ncell + c] with c = j*nx + i (x fastest),
 * v = 0..3 (rho, rho*u, rho*v, E) for 2D.  Mode m <-> (a,b) degrees in (x,y) in the
 * graded order produced by orc_modes().
 */
#ifndef WB_ORACLE_H
#define WB_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BASIS_Q = 0, ORC_BASIS_P = 1 };
enum { ORC_BC_PERIODIC = 0, ORC_BC_COPY = 1 };
enum { ORC_EQ_NONE = 0, ORC_EQ_ISOTHERMAL = 1, ORC_EQ_POLYTROPE = 2 };
enum { ORC_LLF_MAXABS = 0, ORC_LLF_REF2D = 1 };
enum { ORC_RIEMANN_LLF = 0, ORC_RIEMANN_HLLC = 1 };

typedef struct {
  int nx, ny;        /* cells per direction */
  int order;         /* polynomial degree k (0..3) */
  int basis;         /* ORC_BASIS_Q (tensor, (k+1)^2 modes) or ORC_BASIS_P (total degree) */
  int bc_x, bc_y;    /* ORC_BC_* */
  int eq_kind;       /* ORC_EQ_* */
  int llf_speed;     /* ORC_LLF_* wave-speed estimate */
  int limiter;       /* 0 off, 1 minmod moment limiter on the perturbation,
                        2 Zhang-Shu positivity limiter (in delta form) */
  int riemann;       /* ORC_RIEMANN_LLF or ORC_RIEMANN_HLLC */
  double gamma;
  double gx, gy;     /* constant gravity: Phi = gx*x + gy*y */
  double rho0, p0;   /* isothermal: rho = rho0*exp(-(rho0/p0)*Phi), p = p0*exp(-(rho0/p0)*Phi) */
  double kpoly;      /* polytrope: p = K rho^gamma, rho(Phi=0) = 1 */
  double lx, ly;     /* domain [0,lx] x [0,ly] */
  double lim_norm;   /* minmod slope scaling (reference norm = 3) */
  double lim_M;      /* TVB constant: slopes with |norm*s| < M*dx^2 are left alone */
  double lim_tol;    /* a cell is re-limited only if a slope changes by more than this */
  double cfl;
  double pos_eps;    /* positivity floor of density and pressure (reference eps = 1e-10) */
} orc_cfg;

/* perturbation (initial condition) description; shared meaning with the product's */
typedef struct {
  int kind;          /* 0 zero, 1 gaussian pressure bump, 2 multimode velocity */
  int nmodes;        /* kind 2: number of Fourier modes (<= 32) */
  double amp;        /* amplitude */
  double xc, yc;     /* kind 1 centre */
  double sigma;      /* kind 1 width (standard deviation) */
  double kx[32], ky[32], phase_u[32], phase_v[32], weight[32];
} orc_ic;

/* ---- basis / quadrature (2d/legendre.f90) ---- */
double orc_legendre(double x, int n);
double orc_legendre_prime(double x, int n);
void orc_gl_quadrature(int n, double *x, double *w);
int orc_nb(int order, int basis);
int orc_modes(int order, int basis, int *ma, int *mb);

/* ---- modal <-> nodal (2d/benchmark_2d_dg.f90:497-592) on SoA, nvar planes ---- */
void orc_nodes_from_modes(const orc_cfg *c, int nvar, const double *modes, double *nodes);
void orc_modes_from_nodes(const orc_cfg *c, int nvar, const double *nodes, double *modes);

/* ---- equilibrium ---- */
void orc_eq_point(const orc_cfg *c, double ex, double ey, double sx, double sy,
                  double *rho, double *p);
void orc_eq_at(const orc_cfg *c, double x, double y, double *rho, double *p);

/* ---- splitmix64 seeded draws ---- */
uint64_t orc_splitmix64(uint64_t *state);
double orc_uniform(uint64_t *state);

/* ---- initial perturbation, projected to modes ---- */
void orc_project_ic(const orc_cfg *c, const orc_ic *ic, double *delta);

/* ---- the composed 2D well-balanced DG operator, FP64 literal delta-split ---- */
void orc_rhs(const orc_cfg *c, const double *delta, double *dudt);
void orc_limit(const orc_cfg *c, const double *in, double *out);
/* Zhang-Shu positivity limiter in delta form: compute_positivity (2d/limiters.f90:478-654)
 * applied to the full-state polynomial e + delta (e = the cell's projected equilibrium);
 * writes delta back.  Cells left untouched by the limiter are copied bit for bit. */
void orc_positivity(const orc_cfg *c, const double *in, double *out);
/* The literal compute_positivity on full-state modes (SoA, this file's mode order).
 * ref_gll_nodes != 0 takes the reference's two-point GLL node list {-1, 0}
 * (2d/legendre.f90:122-126) for degree 1; 0 takes the Lobatto nodes {-1, +1}.
 * theta_out / t_out (may be NULL) receive each cell's density and pressure factors. */
void orc_ref_positivity(const orc_cfg *c, const double *u_in, double *u_out,
                        int ref_gll_nodes, double *theta_out, double *t_out);
/* solve_for_t, 2d/limiters.f90:312-362 (u and u_avg: rho, mx, my, E) */
double orc_solve_for_t(const orc_cfg *c, const double *u, const double *u_avg);
/* Projected equilibrium (rho and E modes) of cell (i, j): get_modes_from_nodes
 * (2d/benchmark_2d_dg.f90:497-542) of the equilibrium at the GL points. */
void orc_eq_modes(const orc_cfg *c, int i, int j, double *e_rho, double *e_E);
void orc_max_speed(const orc_cfg *c, const double *delta, double *smax_x, double *smax_y);
double orc_cfl_dt(const orc_cfg *c, double smax_x, double smax_y);
/* nsteps SSP-RK2 steps; dt_fixed > 0 uses that dt, else CFL dt each step.
 * The state is limited once before the first step (as evolve does); returns final t. */
double orc_run_rk2(const orc_cfg *c, double *delta, int nsteps, double dt_fixed);
/* SSP-RK(5,4) steps with the coefficients of 2d/benchmark_2d_dg.f90:683-710 */
double orc_run_rk54(const orc_cfg *c, double *delta, int nsteps, double dt_fixed);
void orc_norms(const orc_cfg *c, const double *a, const double *b, double *l1, double *linf,
               double *l2);
void orc_set_threads(int n);
int orc_get_threads(void);

/* ---- literal restatement of the reference 2D DG operator (plain, non-WB) ----
 * 2d/benchmark_2d_dg.f90:1137-1479 with its Fortran layout u(nvar,nx,ny,mx,my),
 * column-major.  ref_flux_bug=1 reproduces flux_type='llf' never matching 'llf1'
 * (face fluxes stay zero); ref_source selects get_source (2) or none (1);
 * grad_phi_bug=1 reproduces grad_phi case 1 (grad = (x,y)) with the '+' sign. */
void orc_ref2d_compute_update(int nx, int ny, int m, double gamma, double lx, double ly,
                              int ref_flux_bug, int ref_source, int grad_phi_bug,
                              double gx, double gy, int bc,
                              const double *u, double *dudt);

/* ---- literal restatement of the reference 1D WB DG operator ----
 * dg_with_source.f90:1749-2031 (compute_update_exact_delta) with LLF (riemann=1),
 * equilibrium rho=p=exp(-x), periodic face indexing of the interior faces and the
 * end-cell freeze of :2028-2029.  half_source=1 keeps the 0.5 on the source
 * projection (as :1998-2006 do).  Layout u(nvar=3, n, nx) column-major. */
void orc_dg1d_update_exact_delta(int nx, int n, double gamma, double lx, int half_source,
                                 int riemann, const double *delta_u, double *dudt);
/* (riemann above is the reference's own switch: 1 riemann_llf, 2 riemann_hllc) */
/* riemann_hllc, dg_with_source.f90:1318-1374 (1D, u = (rho, rho u, E)), literal */
void orc_ref_riemann_hllc(double gamma, const double *ul, const double *ur, double *f);
/* The composed scheme's numerical flux of 2D states in direction dir (0 x, 1 y):
 * LLF or HLLC as cfg->riemann says */
void orc_num_flux(const orc_cfg *c, const double *uL, const double *uR, int dir, double *f);

/* ---- 1D well-balanced FV (benchmark_1d.f90:263-377) with minmod MUSCL on delta ---- */
typedef struct {
  int nx;
  int bc;            /* 0 periodic, 1 equilibrium-extrapolated (copy delta) */
  int limiter;       /* 0 first order, 1 minmod MUSCL on delta */
  int eq_kind;       /* ORC_EQ_ISOTHERMAL / ORC_EQ_POLYTROPE */
  int scheme;        /* 0 'EQL' (equilibrium + delta faces), 1 'WB1' (hydrostatic reconstruction) */
  int pad0;
  double gamma, g, rho0, p0, kpoly, lx, cfl;
} orc_fv1d_cfg;
void orc_fv1d_rhs(const orc_fv1d_cfg *c, const double *delta, double *dudt);
double orc_fv1d_run(const orc_fv1d_cfg *c, double *delta, double tend, int max_steps,
                    int *steps_done);
void orc_fv1d_eq_cells(const orc_fv1d_cfg *c, double *rho, double *p);

#ifdef __cplusplus
}
#endif
#endif
