/* A plain C consumer of libhexagpu.so: the boundary exercised with no Python
 * and no torch, as a foreign-language host (Julia's ccall, cgo, JNI) sees it.
 * Without arguments it checks the host-only entry points and that a context
 * either opens or reports HEXA_ERR_NO_DEVICE; with "gpu" it also runs a small
 * mixed and FP64 solve, the filter and the density update on device 0.
 * Exit status 0 and a final "ok" line mean every check passed. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hexagpu.h"

#define CHECK(cond, code)                                   \
  do {                                                      \
    if (!(cond)) {                                          \
      fprintf(stderr, "check failed (%d): %s\n", code, #cond); \
      return code;                                          \
    }                                                       \
  } while (0)

static int host_checks(void) {
  hexa_solve_params p;
  hexa_default_params(&p);
  CHECK(p.tol == 1e-9 && p.precond == HEXA_PRECOND_MULTIGRID && p.max_iter > 0, 10);
  double ke[576];
  CHECK(hexa_canonical_stiffness(1.0, 1.0, 1.0, 0.3, ke) == HEXA_OK, 11);
  for (int i = 0; i < 24; ++i) {
    double row = 0.0;
    for (int j = 0; j < 24; ++j) {
      CHECK(fabs(ke[i * 24 + j] - ke[j * 24 + i]) <= 1e-14 * fabs(ke[i * 24 + i]), 12); /* symmetric */
      if (j % 3 == 0) row += ke[i * 24 + j];                                            /* x translation */
    }
    CHECK(fabs(row) <= 1e-12, 13); /* a rigid translation is in the null space */
  }
  CHECK(hexa_canonical_stiffness(-1.0, 1.0, 1.0, 0.3, ke) == HEXA_ERR_ARG, 14);
  double kes[64], mes[64];
  CHECK(hexa_scalar_canonical_matrices(1.0, 1.0, 1.0, 0, kes, mes) == HEXA_OK, 15);
  double msum = 0.0;
  for (int i = 0; i < 64; ++i) msum += mes[i];
  CHECK(fabs(msum - 1.0) <= 1e-13, 16); /* the consistent mass of a unit brick sums to its volume */
  hexa_density_update_params up;
  hexa_default_density_update_params(&up);
  CHECK(up.filter_max_iter == 200 && up.filter_precision == HEXA_PREC_FP32 && up.hard_update == 0, 17);
  CHECK(hexa_version() > 0, 18);
  return 0;
}

static int gpu_checks(hexa_ctx* ctx) {
  const hexa_grid g = {16, 8, 8, 1.0, 1.0, 1.0};
  const long ne = 16L * 8 * 8, nn = 17L * 9 * 9, ndof = 3 * nn;
  double* fac = malloc(sizeof(double) * ne);
  double* f = calloc(ndof, sizeof(double));
  double* u32 = malloc(sizeof(double) * ndof);
  double* u64 = malloc(sizeof(double) * ndof);
  CHECK(fac && f && u32 && u64, 20);
  for (long e = 0; e < ne; ++e) {
    const double rho = 0.2 + 0.8 * (double)((e * 7919) % 101) / 100.0;
    fac[e] = 1e-9 + rho * rho * rho * (1.0 - 1e-9);
  }
  for (long j = 0; j <= 8; ++j) f[3 * (16 + 17 * j) + 2] = -1.0 / 9.0; /* the x = max, z = 0 edge */
  const hexa_bc bc = {1u, NULL};                                     /* x = 0 face clamped */
  hexa_solve_params p;
  hexa_default_params(&p);
  p.divergence_check = 0;
  hexa_solve_stats s32, s64;
  p.precision = HEXA_PREC_MIXED;
  CHECK(hexa_solve(ctx, &g, &bc, fac, f, &p, NULL, u32, &s32) == HEXA_OK, 21);
  p.precision = HEXA_PREC_FP64;
  p.tol = 1e-12;
  CHECK(hexa_solve(ctx, &g, &bc, fac, f, &p, NULL, u64, &s64) == HEXA_OK, 22);
  CHECK(s32.true_relres <= 1e-9 && s64.true_relres <= 1e-12, 23);
  double d = 0.0, n = 0.0;
  for (long i = 0; i < ndof; ++i) d += (u32[i] - u64[i]) * (u32[i] - u64[i]), n += u64[i] * u64[i];
  CHECK(n > 0.0 && sqrt(d / n) <= 1e-7, 24);
  CHECK(fabs(s32.compliance - s64.compliance) <= 1e-8 * fabs(s64.compliance), 25);
  /* the true-brick filter keeps a constant field */
  double* rho = malloc(sizeof(double) * ne);
  double* out = malloc(sizeof(double) * ne);
  CHECK(rho && out, 26);
  for (long e = 0; e < ne; ++e) rho[e] = 0.4;
  hexa_filter_stats fs;
  CHECK(hexa_filter(ctx, &g, rho, 1.5, 1e-10, 400, 0, HEXA_PREC_FP64, out, &fs) == HEXA_OK, 27);
  for (long e = 0; e < ne; ++e) CHECK(fabs(out[e] - 0.4) <= 1e-8, 28);
  /* the density update: a uniform stress ratio gives a uniform density */
  float* dens = malloc(sizeof(float) * ne);
  float* l1 = malloc(sizeof(float) * ne);
  float* orig = malloc(sizeof(float) * ne);
  CHECK(dens && l1 && orig, 29);
  for (long e = 0; e < ne; ++e) dens[e] = 0.5f, l1[e] = 60.0f, orig[e] = 1.0f;
  hexa_density_update_params up;
  hexa_default_density_update_params(&up);
  up.E = 100.0f;
  up.iter = 1;
  up.max_domain_dim = 16.0f;
  up.minimum_filter_radius_as_elements = 0.0f;
  hexa_density_update_stats us;
  CHECK(hexa_update_density(ctx, &g, dens, l1, NULL, orig, &up, &us) == HEXA_OK, 30);
  CHECK(us.status == 0 && us.filter_used == 0 && us.culled == 0 && us.active_count == ne, 31);
  for (long e = 0; e < ne; ++e) CHECK(dens[e] == 0.6f, 32);
  /* Solver.solve_system with the reference's argument types: a void block of
   * 4x4x2 elements (density at the minimum, 3 % of the 1024) is pruned from
   * outer iteration 3 on; its interior nodes get u = 0 (reconstruct_full_solution) */
  float* dens32 = malloc(sizeof(float) * ne);
  float* f32 = calloc(ndof, sizeof(float));
  float* bcind = calloc(ndof, sizeof(float)); /* Matrix{Float32}(nNodes, 3), column-major */
  CHECK(dens32 && f32 && bcind, 35);
  for (long e = 0; e < ne; ++e) {
    const long i = e % 16, j = (e / 16) % 8, k = e / 128;
    dens32[e] = (i >= 6 && i < 10 && j >= 2 && j < 6 && k >= 2 && k < 4) ? 1e-3f : 0.5f;
  }
  for (long nd = 0; nd < nn; ++nd)
    if (nd % 17 == 0)
      for (int c = 0; c < 3; ++c) bcind[nd + nn * c] = 1.0f;
  for (long j = 0; j <= 8; ++j) f32[3 * (16 + 17 * j) + 2] = -1.0f / 9.0f;
  hexa_solve_params ps;
  hexa_default_params(&ps);
  ps.tol = 1e-10;
  ps.divergence_check = 0;
  double relres = 1.0;
  char name[32];
  int64_t active = 0;
  hexa_solve_stats ss;
  CHECK(hexa_solve_system(ctx, &g, 1.0f, bcind, f32, dens32, 1e-3f, 1, 3, &ps, NULL, u64, &relres, name, 32, &ss,
                          &active) == HEXA_OK, 36);
  CHECK(active == ne - 32, 37);
  CHECK(ss.true_relres <= 1e-10, 43);
  CHECK(strcmp(name, "GMG_GPU") == 0, 44);
  const long mid = 8 + 17 * (4 + 9 * 3); /* a node inside the void block */
  CHECK(u64[3 * mid] == 0.0 && u64[3 * mid + 1] == 0.0 && u64[3 * mid + 2] == 0.0, 38);
  CHECK(u64[3 * (mid + 5) + 2] != 0.0, 45); /* a node outside it moves */
  CHECK(hexa_solve_system(ctx, &g, 1.0f, bcind, f32, dens32, 1e-3f, 1, 2, &ps, NULL, u64, &relres, name, 32, &ss,
                          &active) == HEXA_OK && active == ne, 39);
  free(dens32), free(f32), free(bcind);
  CHECK(hexa_solve(ctx, NULL, &bc, fac, f, &p, NULL, u64, &s64) == HEXA_ERR_ARG, 33);
  CHECK(strlen(hexa_last_error(ctx)) > 0, 34);
  free(fac), free(f), free(u32), free(u64), free(rho), free(out), free(dens), free(l1), free(orig);
  return 0;
}

int main(int argc, char** argv) {
  const int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
  int rc = host_checks();
  if (rc) return rc;
  hexa_ctx* ctx = NULL;
  const int cr = hexa_create(0, &ctx);
  if (gpu) {
    CHECK(cr == HEXA_OK && ctx, 40);
    rc = gpu_checks(ctx);
    hexa_destroy(ctx);
    if (rc) return rc;
  } else {
    CHECK(cr == HEXA_OK || cr == HEXA_ERR_NO_DEVICE, 41);
    CHECK((cr == HEXA_OK) == (ctx != NULL), 42);
    if (ctx) hexa_destroy(ctx);
  }
  printf("ok %s\n", gpu ? "gpu" : "host");
  return 0;
}
