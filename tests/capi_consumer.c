/*
 * capi_consumer.c -- a C program compiled against include/wb_capi.h and linked to
 * libwbgb300.so, standing in for the reference's Fortran driver (no Fortran compiler is
 * available to build the ISO_C_BINDING module).  Built and run by tests/test_capi_consumer.py.
 *
 *   capi_consumer layout
 *       prints sizeof / offsetof of every struct the ABI passes, as one JSON object
 *       (the test checks them against the ctypes mirrors);
 *   capi_consumer evolve IN OUT OUT2 NX NY ORDER TEND
 *       the shape of evolve (2d/benchmark_2d_dg.f90:624-775) over the ABI: configuration
 *       from the defaults, the Fortran-layout state u(4, nx, ny, k+1, k+1) read from IN
 *       (raw doubles, column-major), wb_max_speed (compute_max_speed, :826-870), wb_evolve
 *       to TEND, wb_download_state into OUT, wb_norms (compute_error, :23-89), then two
 *       fixed wb_step steps + wb_sync, downloaded into OUT2; one JSON line on stdout.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

#include "wb_capi.h"

#define FIELD(T, f) printf("\"%s.%s\": %zu, ", #T, #f, offsetof(T, f))

static int layout(void) {
  printf("{");
  printf("\"wb_config\": %zu, ", sizeof(wb_config));
  FIELD(wb_config, nx); FIELD(wb_config, ny); FIELD(wb_config, order); FIELD(wb_config, basis);
  FIELD(wb_config, bc_x); FIELD(wb_config, bc_y); FIELD(wb_config, eq_kind);
  FIELD(wb_config, llf_speed); FIELD(wb_config, limiter); FIELD(wb_config, precision);
  FIELD(wb_config, integrator); FIELD(wb_config, tile_x); FIELD(wb_config, tile_y);
  FIELD(wb_config, device); FIELD(wb_config, riemann); FIELD(wb_config, cells_per_thread);
  FIELD(wb_config, gamma); FIELD(wb_config, gx); FIELD(wb_config, gy); FIELD(wb_config, rho0);
  FIELD(wb_config, p0); FIELD(wb_config, kpoly); FIELD(wb_config, lx); FIELD(wb_config, ly);
  FIELD(wb_config, lim_norm); FIELD(wb_config, lim_M); FIELD(wb_config, lim_tol);
  FIELD(wb_config, cfl); FIELD(wb_config, pos_eps);
  printf("\"wb_perturbation\": %zu, ", sizeof(wb_perturbation));
  FIELD(wb_perturbation, kind); FIELD(wb_perturbation, nmodes); FIELD(wb_perturbation, amp);
  FIELD(wb_perturbation, xc); FIELD(wb_perturbation, yc); FIELD(wb_perturbation, sigma);
  FIELD(wb_perturbation, kx); FIELD(wb_perturbation, ky); FIELD(wb_perturbation, phase_u);
  FIELD(wb_perturbation, phase_v); FIELD(wb_perturbation, weight);
  printf("\"wb1d_config\": %zu, ", sizeof(wb1d_config));
  FIELD(wb1d_config, nx); FIELD(wb1d_config, bc); FIELD(wb1d_config, limiter);
  FIELD(wb1d_config, eq_kind); FIELD(wb1d_config, device); FIELD(wb1d_config, scheme);
  FIELD(wb1d_config, gamma); FIELD(wb1d_config, g); FIELD(wb1d_config, rho0);
  FIELD(wb1d_config, p0); FIELD(wb1d_config, kpoly); FIELD(wb1d_config, lx);
  printf("\"wb1d_config.cfl\": %zu}\n", offsetof(wb1d_config, cfl));
  return 0;
}

static int fail(wb_ctx *ctx, const char *what, int rc) {
  fprintf(stderr, "%s: %s (%d): %s\n", what, wb_status_string(rc), rc,
          ctx ? wb_last_error(ctx) : "");
  if (ctx) wb_destroy(ctx);
  return 1;
}

static int io(const char *path, double *a, size_t n, int write) {
  FILE *f = fopen(path, write ? "wb" : "rb");
  if (!f) return -1;
  size_t k = write ? fwrite(a, sizeof(double), n, f) : fread(a, sizeof(double), n, f);
  fclose(f);
  return k == n ? 0 : -1;
}

static int evolve(const char *in, const char *out, const char *out2, int nx, int ny, int order,
                  double tend) {
  wb_config cfg;
  int rc = wb_config_default(&cfg);
  if (rc) return fail(NULL, "wb_config_default", rc);
  cfg.nx = nx;
  cfg.ny = ny;
  cfg.order = order;
  cfg.basis = WB_BASIS_Q; /* the reference's tensor basis: the Fortran layout needs it */
  cfg.bc_x = WB_BC_COPY;
  cfg.bc_y = WB_BC_COPY;
  cfg.eq_kind = WB_EQ_ISOTHERMAL;
  cfg.gx = 1.0;
  cfg.gy = 1.0;
  cfg.limiter = WB_LIMITER_MINMOD;
  cfg.precision = WB_PREC_FP64;
  cfg.integrator = WB_RK2;
  cfg.cfl = 0.3;
  const size_t n = (size_t)4 * nx * ny * (order + 1) * (order + 1);
  double *u = malloc(n * sizeof(double));
  if (!u || io(in, u, n, 0)) {
    fprintf(stderr, "cannot read %s\n", in);
    return 1;
  }
  wb_ctx *ctx = NULL;
  if ((rc = wb_create(&cfg, &ctx))) return fail(ctx, "wb_create", rc);
  if ((rc = wb_upload_state(ctx, u, WB_LAYOUT_FORTRAN))) return fail(ctx, "wb_upload_state", rc);
  double sx = 0.0, sy = 0.0;
  if ((rc = wb_max_speed(ctx, &sx, &sy))) return fail(ctx, "wb_max_speed", rc);
  int32_t steps = 0;
  double t = 0.0;
  if ((rc = wb_evolve(ctx, tend, 1 << 30, &steps, &t))) return fail(ctx, "wb_evolve", rc);
  if ((rc = wb_download_state(ctx, u, WB_LAYOUT_FORTRAN))) return fail(ctx, "wb_download_state", rc);
  if (io(out, u, n, 1)) return fail(ctx, "write OUT", WB_ERR_ARG);
  double l1[4], linf[4], l2[4];
  if ((rc = wb_norms(ctx, NULL, l1, linf, l2))) return fail(ctx, "wb_norms", rc);
  if ((rc = wb_step(ctx, 2, 1e-4))) return fail(ctx, "wb_step", rc);
  if ((rc = wb_sync(ctx))) return fail(ctx, "wb_sync", rc);
  if ((rc = wb_download_state(ctx, u, WB_LAYOUT_FORTRAN))) return fail(ctx, "wb_download_state", rc);
  if (io(out2, u, n, 1)) return fail(ctx, "write OUT2", WB_ERR_ARG);
  double t2 = 0.0;
  int64_t steps2 = 0;
  if ((rc = wb_get_time(ctx, &t2, &steps2))) return fail(ctx, "wb_get_time", rc);
  printf("{\"steps\": %d, \"t\": %.17g, \"smax\": [%.17g, %.17g], \"l1\": [%.17g, %.17g, %.17g, %.17g], "
         "\"linf\": [%.17g, %.17g, %.17g, %.17g], \"t2\": %.17g, \"steps2\": %lld}\n",
         steps, t, sx, sy, l1[0], l1[1], l1[2], l1[3], linf[0], linf[1], linf[2], linf[3], t2,
         (long long)steps2);
  wb_destroy(ctx);
  free(u);
  return 0;
}

int main(int argc, char **argv) {
  if (argc == 2 && argv[1][0] == 'l') return layout();
  if (argc == 9 && argv[1][0] == 'e')
    return evolve(argv[2], argv[3], argv[4], atoi(argv[5]), atoi(argv[6]), atoi(argv[7]),
                  atof(argv[8]));
  fprintf(stderr, "usage: %s layout | evolve IN OUT OUT2 NX NY ORDER TEND\n", argv[0]);
  return 2;
}
