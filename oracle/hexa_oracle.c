/*
 * hexa_oracle.c -- CPU restatement of the reference's FE-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker and the timed
 * CPU baseline; the GPU library never links or calls it.  Each function
 * restates the reference file:lines named in its comment, written as plain
 * element loops in the reference's order (element scatter, node-major DOFs),
 * in FP64 unless stated.
 *
 * Layout: node (i,j,k) 0-based -> i + (nx+1)*(j + (ny+1)*k); element
 * e = i + nx*(j + ny*k); local nodes n1..n8 as src/Mesh/Mesh.jl:45-53.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const int NAT[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
/* offsets of n1..n8 from the element's min corner (Mesh.jl:45-53) */
static const int OFF[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

static void elem_nodes(int nx, int ny, long long e, long long n[8]) {
  const long long NX = nx + 1, NY = ny + 1;
  const long long i = e % nx, t = e / nx, j = t % ny, k = t / ny;
  for (int a = 0; a < 8; ++a) n[a] = (i + OFF[a][0]) + NX * ((j + OFF[a][1]) + NY * (k + OFF[a][2]));
}

/* ---------------------------------------------------------------------------
 * Element.jl:23-111 -- shape_functions, material_matrix, hex_element_stiffness,
 * get_canonical_stiffness.  fp32 != 0 evaluates every step in float (the
 * reference's element type); otherwise in double.  Output 24x24 column-major.
 */
#define KE_BODY(REAL)                                                                                 \
  {                                                                                                   \
    REAL nodes[8][3] = {{0, 0, 0}, {dx, 0, 0}, {dx, dy, 0}, {0, dy, 0},                               \
                        {0, 0, dz}, {dx, 0, dz}, {dx, dy, dz}, {0, dy, dz}};                          \
    for (int a = 0; a < 8; ++a) {                                                                     \
      nodes[a][0] -= (REAL)dx / 2; nodes[a][1] -= (REAL)dy / 2; nodes[a][2] -= (REAL)dz / 2;          \
    }                                                                                                 \
    const REAL one = 1, two = 2;                                                                      \
    const REAL inv_den = one / ((one + (REAL)nu) * (one - two * (REAL)nu));                           \
    const REAL c1 = (one - (REAL)nu) * inv_den, c2 = (REAL)nu * inv_den;                             \
    const REAL c3 = ((one - two * (REAL)nu) / two) * inv_den;                                        \
    REAL D[6][6] = {{0}};                                                                             \
    D[0][0] = D[1][1] = D[2][2] = c1;                                                                 \
    D[0][1] = D[0][2] = D[1][0] = D[1][2] = D[2][0] = D[2][1] = c2;                                   \
    D[3][3] = D[4][4] = D[5][5] = c3;                                                                 \
    REAL ke[24][24] = {{0}};                                                                          \
    const REAL ga = one / (REAL)sqrt((REAL)3);                                                       \
    const REAL gp[2] = {-ga, ga};                                                                     \
    for (int ix = 0; ix < 2; ++ix)                                                                    \
      for (int iy = 0; iy < 2; ++iy)                                                                  \
        for (int iz = 0; iz < 2; ++iz) {                                                              \
          const REAL xi = gp[ix], eta = gp[iy], zeta = gp[iz];                                        \
          REAL dN[8][3];                                                                              \
          for (int a = 0; a < 8; ++a) {                                                               \
            const REAL tx = one + xi * NAT[a][0], ty = one + eta * NAT[a][1], tz = one + zeta * NAT[a][2]; \
            dN[a][0] = (REAL)0.125 * NAT[a][0] * ty * tz;                                            \
            dN[a][1] = (REAL)0.125 * tx * NAT[a][1] * tz;                                            \
            dN[a][2] = (REAL)0.125 * tx * ty * NAT[a][2];                                            \
          }                                                                                           \
          REAL J[3][3] = {{0}};                                                                       \
          for (int r = 0; r < 3; ++r)                                                                 \
            for (int s = 0; s < 3; ++s)                                                               \
              for (int a = 0; a < 8; ++a) J[r][s] += dN[a][r] * nodes[a][s];                         \
          const REAL det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -                        \
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +                        \
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);                         \
          if (!(det > 0)) return -2;                                                                  \
          REAL Ji[3][3];                                                                              \
          Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;                                   \
          Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;                                   \
          Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;                                   \
          Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;                                   \
          Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;                                   \
          Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;                                   \
          Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;                                   \
          Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;                                   \
          Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;                                   \
          REAL G[8][3];                                                                               \
          for (int a = 0; a < 8; ++a)                                                                 \
            for (int r = 0; r < 3; ++r) {                                                             \
              REAL s = 0;                                                                             \
              for (int q = 0; q < 3; ++q) s += dN[a][q] * Ji[r][q];                                   \
              G[a][r] = s;                                                                            \
            }                                                                                         \
          REAL B[6][24] = {{0}};                                                                      \
          for (int a = 0; a < 8; ++a) {                                                               \
            const int o = 3 * a;                                                                      \
            B[0][o] = G[a][0]; B[1][o + 1] = G[a][1]; B[2][o + 2] = G[a][2];                          \
            B[3][o] = G[a][1]; B[3][o + 1] = G[a][0];                                                 \
            B[4][o + 1] = G[a][2]; B[4][o + 2] = G[a][1];                                             \
            B[5][o] = G[a][2]; B[5][o + 2] = G[a][0];                                                 \
          }                                                                                           \
          for (int r = 0; r < 24; ++r)                                                                \
            for (int c = 0; c < 24; ++c) {                                                            \
              REAL s = 0;                                                                             \
              for (int p = 0; p < 6; ++p)                                                             \
                for (int q = 0; q < 6; ++q) s += B[p][r] * D[p][q] * B[q][c];                         \
              ke[r][c] += s * det;                                                                    \
            }                                                                                         \
        }                                                                                             \
    for (int r = 0; r < 24; ++r)                                                                      \
      for (int c = 0; c < 24; ++c) out[r + 24 * c] = (double)ke[r][c];                                \
    return 0;                                                                                         \
  }

static int ke_double(double dx, double dy, double dz, double nu, double* out) KE_BODY(double)
static int ke_float(float dx, float dy, float dz, float nu, double* out) KE_BODY(float)

int ho_canonical_stiffness(double dx, double dy, double dz, double nu, int fp32, double* out) {
  if (fp32) return ke_float((float)dx, (float)dy, (float)dz, (float)nu, out);
  return ke_double(dx, dy, dz, nu, out);
}

/* Element.jl:113-134 -- scalar Laplacian Ke and mass Me; quirk = top z at +dz. */
int ho_scalar_matrices(double dx, double dy, double dz, int quirk, double* Ke, double* Me) {
  const double zt = quirk ? dz : dz / 2;
  const double nodes[8][3] = {{-dx / 2, -dy / 2, -dz / 2}, {dx / 2, -dy / 2, -dz / 2}, {dx / 2, dy / 2, -dz / 2},
                              {-dx / 2, dy / 2, -dz / 2},  {-dx / 2, -dy / 2, zt},    {dx / 2, -dy / 2, zt},
                              {dx / 2, dy / 2, zt},        {-dx / 2, dy / 2, zt}};
  memset(Ke, 0, 64 * sizeof(double));
  memset(Me, 0, 64 * sizeof(double));
  const double ga = 1.0 / sqrt(3.0), gp[2] = {-ga, ga};
  for (int ix = 0; ix < 2; ++ix)
    for (int iy = 0; iy < 2; ++iy)
      for (int iz = 0; iz < 2; ++iz) {
        double N[8], dN[8][3];
        for (int a = 0; a < 8; ++a) {
          const double tx = 1 + gp[ix] * NAT[a][0], ty = 1 + gp[iy] * NAT[a][1], tz = 1 + gp[iz] * NAT[a][2];
          N[a] = 0.125 * tx * ty * tz;
          dN[a][0] = 0.125 * NAT[a][0] * ty * tz;
          dN[a][1] = 0.125 * tx * NAT[a][1] * tz;
          dN[a][2] = 0.125 * tx * ty * NAT[a][2];
        }
        double J[3][3] = {{0}};
        for (int r = 0; r < 3; ++r)
          for (int s = 0; s < 3; ++s)
            for (int a = 0; a < 8; ++a) J[r][s] += dN[a][r] * nodes[a][s];
        /* the brick's Jacobian is diagonal */
        const double det = J[0][0] * J[1][1] * J[2][2];
        double G[8][3];
        for (int a = 0; a < 8; ++a)
          for (int r = 0; r < 3; ++r) G[a][r] = dN[a][r] / J[r][r];
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) {
            Ke[r + 8 * c] += (G[r][0] * G[c][0] + G[r][1] * G[c][1] + G[r][2] * G[c][2]) * det;
            Me[r + 8 * c] += N[r] * N[c] * det;
          }
      }
  return 0;
}

/* ---------------------------------------------------------------------------
 * GPUSolver.jl:91-128 (matvec_unstructured_atomic_kernel!) as a sequential
 * element scatter: y = sum_e factor_e * K0 * u_e over the full DOF vector.
 * Parallel over z-slabs of elements with private accumulation: each thread
 * owns whole element layers of one colour (even / odd k), so no two threads
 * write one node at the same time and the result is deterministic.
 */
void ho_apply_K(int nx, int ny, int nz, const double* K0, const double* factor, const double* x, double* y) {
  const long long NX = nx + 1, NY = ny + 1, NZ = nz + 1;
  memset(y, 0, sizeof(double) * 3 * NX * NY * NZ);
  for (int parity = 0; parity < 2; ++parity) {
#pragma omp parallel for schedule(static)
    for (int k = parity; k < nz; k += 2) {
      for (long long e = (long long)k * nx * ny; e < (long long)(k + 1) * nx * ny; ++e) {
        long long n[8];
        elem_nodes(nx, ny, e, n);
        double ue[24], fe[24];
        for (int a = 0; a < 8; ++a)
          for (int c = 0; c < 3; ++c) ue[3 * a + c] = x[3 * n[a] + c];
        for (int r = 0; r < 24; ++r) {
          double s = 0.0;
          for (int c = 0; c < 24; ++c) s += K0[r + 24 * c] * ue[c];
          fe[r] = s * factor[e];
        }
        for (int a = 0; a < 8; ++a)
          for (int c = 0; c < 3; ++c) y[3 * n[a] + c] += fe[3 * a + c];
      }
    }
  }
}

/* GPUSolver.jl:130-144: diag of K with the x-diagonal of K0 for all three
 * components (quirk = 1) or the component's own diagonal (quirk = 0). */
void ho_diag_K(int nx, int ny, int nz, const double* K0, const double* factor, int quirk, double* d) {
  const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  memset(d, 0, sizeof(double) * 3 * nn);
  const long long ne = (long long)nx * ny * nz;
  for (long long e = 0; e < ne; ++e) {
    long long n[8];
    elem_nodes(nx, ny, e, n);
    for (int a = 0; a < 8; ++a)
      for (int c = 0; c < 3; ++c) {
        const int l = quirk ? 3 * a : 3 * a + c;
        d[3 * n[a] + c] += K0[l + 24 * l] * factor[e];
      }
  }
}

/* u_e^T K0 u_e per element (sensitivity numerator). */
void ho_element_energy(int nx, int ny, int nz, const double* K0, const double* u, double* ce) {
  const long long ne = (long long)nx * ny * nz;
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < ne; ++e) {
    long long n[8];
    elem_nodes(nx, ny, e, n);
    double ue[24];
    for (int a = 0; a < 8; ++a)
      for (int c = 0; c < 3; ++c) ue[3 * a + c] = u[3 * n[a] + c];
    double s = 0.0;
    for (int r = 0; r < 24; ++r) {
      double t = 0.0;
      for (int c = 0; c < 24; ++c) t += K0[r + 24 * c] * ue[c];
      s += ue[r] * t;
    }
    ce[e] = s;
  }
}

/* GPUHelmholtz.jl:73-97 / TopOpt.jl:32-79: y = sum_e Ae x_e, Ae 8x8 column-major
 * in n1..n8 order; parity colouring over k as in ho_apply_K. */
void ho_helm_apply(int nx, int ny, int nz, const double* Ae, const double* x, double* y) {
  const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  memset(y, 0, sizeof(double) * nn);
  for (int parity = 0; parity < 2; ++parity) {
#pragma omp parallel for schedule(static)
    for (int k = parity; k < nz; k += 2) {
      for (long long e = (long long)k * nx * ny; e < (long long)(k + 1) * nx * ny; ++e) {
        long long n[8];
        elem_nodes(nx, ny, e, n);
        double xe[8];
        for (int a = 0; a < 8; ++a) xe[a] = x[n[a]];
        for (int r = 0; r < 8; ++r) {
          double s = 0.0;
          for (int c = 0; c < 8; ++c) s += Ae[r + 8 * c] * xe[c];
          y[n[r]] += s;
        }
      }
    }
  }
}

/* GPUHelmholtz.jl:59-70 (RHS) and :99-110 (element mean). */
void ho_helm_rhs(int nx, int ny, int nz, const double* rho, double scale, double* b) {
  const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1), ne = (long long)nx * ny * nz;
  memset(b, 0, sizeof(double) * nn);
  for (long long e = 0; e < ne; ++e) {
    long long n[8];
    elem_nodes(nx, ny, e, n);
    for (int a = 0; a < 8; ++a) b[n[a]] += rho[e] * scale;
  }
}
void ho_helm_extract(int nx, int ny, int nz, const double* psi, double* out) {
  const long long ne = (long long)nx * ny * nz;
  for (long long e = 0; e < ne; ++e) {
    long long n[8];
    elem_nodes(nx, ny, e, n);
    double s = 0.0;
    for (int a = 0; a < 8; ++a) s += psi[n[a]];
    out[e] = s / 8.0;
  }
}

/* GPUHelmholtz.jl:190-266 (solve_helmholtz_on_gpu) on the host in FP64:
 * Jacobi-PCG of (R^2 Ke + Me) psi = sum_e rho_e vol/8, the recursive
 * ||r||/||b|| tested every 10 iterations, at most max_iter iterations, then
 * the element mean of psi (GPUHelmholtz.jl:99-110).  Ae is the 8x8 element
 * matrix, column-major in n1..n8 order.  A zero right-hand side returns rho
 * unchanged (GPUHelmholtz.jl:203-206).  Returns the iteration count; *relres
 * gets the last tested residual.  Vector passes are OpenMP loops with
 * reductions (the sum order depends on the thread count, as the reference's
 * CUBLAS sums depend on its launch shape). */
int ho_helm_pcg(int nx, int ny, int nz, const double* Ae, const double* rho, double scale, double tol, int max_iter,
                double* out, double* relres) {
  const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1), ne = (long long)nx * ny * nz;
  double* b = (double*)malloc(sizeof(double) * nn);
  double* x = (double*)calloc((size_t)nn, sizeof(double));
  double* r = (double*)malloc(sizeof(double) * nn);
  double* z = (double*)malloc(sizeof(double) * nn);
  double* q = (double*)malloc(sizeof(double) * nn);
  double* pv = (double*)malloc(sizeof(double) * nn);
  double* dinv = (double*)calloc((size_t)nn, sizeof(double));
  int it = 0;
  *relres = 0.0;
  if (!b || !x || !r || !z || !q || !pv || !dinv) {
    it = -1;
    goto done;
  }
  ho_helm_rhs(nx, ny, nz, rho, scale, b);
  for (long long e = 0; e < ne; ++e) { /* assembled diagonal: sum of Ae[a][a] over the node's elements */
    long long n[8];
    elem_nodes(nx, ny, e, n);
    for (int a = 0; a < 8; ++a) dinv[n[a]] += Ae[a + 8 * a];
  }
  double bb = 0.0;
#pragma omp parallel for reduction(+ : bb) schedule(static)
  for (long long i = 0; i < nn; ++i) {
    dinv[i] = 1.0 / dinv[i];
    bb += b[i] * b[i];
  }
  const double nb = sqrt(bb);
  if (nb == 0.0) {
    memcpy(out, rho, sizeof(double) * ne);
    goto done;
  }
  double rz = 0.0;
#pragma omp parallel for reduction(+ : rz) schedule(static)
  for (long long i = 0; i < nn; ++i) {
    r[i] = b[i];
    z[i] = r[i] * dinv[i];
    pv[i] = z[i];
    rz += r[i] * z[i];
  }
  for (it = 1; it <= max_iter; ++it) {
    ho_helm_apply(nx, ny, nz, Ae, pv, q);
    double pq = 0.0;
#pragma omp parallel for reduction(+ : pq) schedule(static)
    for (long long i = 0; i < nn; ++i) pq += pv[i] * q[i];
    const double alpha = rz / pq;
    double rr = 0.0;
#pragma omp parallel for reduction(+ : rr) schedule(static)
    for (long long i = 0; i < nn; ++i) {
      x[i] += alpha * pv[i];
      r[i] -= alpha * q[i];
      rr += r[i] * r[i];
    }
    if (it % 10 == 0) {
      *relres = sqrt(rr) / nb;
      if (*relres < tol) break;
    }
    double rzn = 0.0;
#pragma omp parallel for reduction(+ : rzn) schedule(static)
    for (long long i = 0; i < nn; ++i) {
      z[i] = r[i] * dinv[i];
      rzn += r[i] * z[i];
    }
    const double beta = rzn / rz;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nn; ++i) pv[i] = z[i] + beta * pv[i];
    rz = rzn;
  }
  if (it > max_iter) it = max_iter;
  ho_helm_extract(nx, ny, nz, x, out);
done:
  free(b);
  free(x);
  free(r);
  free(z);
  free(q);
  free(pv);
  free(dinv);
  return it;
}

/* ---------------------------------------------------------------------------
 * CPUSolver.jl:56-255 -- the reference's CPU matrix_free path, in Float32 as
 * the reference runs it (T = Float32 from nodes/E, src/Main.jl:289-294):
 *   apply_stiffness: each of nthreads tasks scatters its element chunk into a
 *   private full-length buffer, skipping elements with density <
 *   min_stiffness_threshold (:82); the buffers are then summed (:114-119);
 *   compute_diagonal_preconditioner: same pattern with K0 diagonals (:142-190);
 *   matrix_free_cg_solve: shift = shift_factor * max(diag_free), Jacobi with
 *   diag clamped to >= shift, ||r||/||f|| tested every iteration (:192-255).
 * fixed_dof: 3*nNodes bytes (nonzero = constrained).  K0 is passed in (FP32
 * values).  Returns the iteration count; *relres, *seconds filled.
 * max_seconds > 0 stops early (bounded sample); *iters_done reports it.
 */
typedef struct {
  int nx, ny, nz, nthreads;
  const float* K0;
  const float* density;
  float E, min_thr;
  const uint8_t* fixed;
  long long ndof;
  long long* free_idx;
  long long nfree;
  float* partial; /* nthreads * ndof */
  float* xfull;
  float* yfull;
} cpu_sys;

static void cpu_apply(cpu_sys* S, const float* x_free, float* y_free) {
  const long long ne = (long long)S->nx * S->ny * S->nz;
  memset(S->xfull, 0, sizeof(float) * S->ndof);
  for (long long i = 0; i < S->nfree; ++i) S->xfull[S->free_idx[i]] = x_free[i];
  const int T = S->nthreads;
  const long long chunk = (ne + T - 1) / T;
#pragma omp parallel for num_threads(T) schedule(static, 1)
  for (int t = 0; t < T; ++t) {
    float* loc = S->partial + (long long)t * S->ndof;
    memset(loc, 0, sizeof(float) * S->ndof);
    const long long e0 = t * chunk, e1 = (e0 + chunk < ne) ? e0 + chunk : ne;
    float ue[24], fe[24];
    for (long long e = e0; e < e1; ++e) {
      const float dens = S->density[e];
      if (!(dens >= S->min_thr)) continue;
      long long n[8];
      elem_nodes(S->nx, S->ny, e, n);
      const float factor = S->E * dens;
      for (int a = 0; a < 8; ++a)
        for (int c = 0; c < 3; ++c) ue[3 * a + c] = S->xfull[3 * n[a] + c];
      for (int r = 0; r < 24; ++r) {
        float s = 0.0f;
        for (int c = 0; c < 24; ++c) s += S->K0[r + 24 * c] * ue[c];
        fe[r] = s * factor;
      }
      for (int a = 0; a < 8; ++a)
        for (int c = 0; c < 3; ++c) loc[3 * n[a] + c] += fe[3 * a + c];
    }
  }
  /* result .+= partial_results (sequential over tasks, parallel over DOFs) */
  float* y = S->yfull;
#pragma omp parallel for num_threads(T) schedule(static)
  for (long long i = 0; i < S->ndof; ++i) {
    float s = 0.0f;
    for (int t = 0; t < T; ++t) s += S->partial[(long long)t * S->ndof + i];
    y[i] = s;
  }
  for (long long i = 0; i < S->nfree; ++i) y_free[i] = y[S->free_idx[i]];
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int ho_cpu_matrix_free_cg(int nx, int ny, int nz, const float* K0, float E, const float* density, const float* f,
                          const uint8_t* fixed, float min_thr, int max_iter, float tol, float shift_factor,
                          int nthreads, double max_seconds, float* x_out, double* relres, double* seconds,
                          int* iters_done) {
  cpu_sys S;
  S.nx = nx; S.ny = ny; S.nz = nz;
  S.nthreads = nthreads > 0 ? nthreads : 1;
  S.K0 = K0; S.density = density; S.E = E; S.min_thr = min_thr; S.fixed = fixed;
  const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  S.ndof = 3 * nn;
  S.free_idx = (long long*)malloc(sizeof(long long) * S.ndof);
  S.nfree = 0;
  for (long long i = 0; i < S.ndof; ++i)
    if (!fixed[i]) S.free_idx[S.nfree++] = i;
  S.partial = (float*)malloc(sizeof(float) * S.ndof * S.nthreads);
  S.xfull = (float*)malloc(sizeof(float) * S.ndof);
  S.yfull = (float*)malloc(sizeof(float) * S.ndof);
  const long long nf = S.nfree;
  float *x = (float*)calloc(nf, sizeof(float)), *r = (float*)malloc(sizeof(float) * nf), *z = (float*)malloc(sizeof(float) * nf),
        *p = (float*)malloc(sizeof(float) * nf), *Ap = (float*)malloc(sizeof(float) * nf), *dg = (float*)malloc(sizeof(float) * nf);
  const double t0 = now_s();
  /* compute_diagonal_preconditioner (:142-190) */
  {
    float* dfull = S.yfull;
    memset(dfull, 0, sizeof(float) * S.ndof);
    const long long ne = (long long)nx * ny * nz;
    for (long long e = 0; e < ne; ++e) {
      const float dens = density[e];
      if (!(dens >= min_thr)) continue;
      long long n[8];
      elem_nodes(nx, ny, e, n);
      const float factor = E * dens;
      for (int a = 0; a < 8; ++a)
        for (int c = 0; c < 3; ++c) dfull[3 * n[a] + c] += K0[(3 * a + c) * 25] * factor;
    }
    for (long long i = 0; i < nf; ++i) dg[i] = dfull[S.free_idx[i]];
  }
  float maxd = 0.0f;
  for (long long i = 0; i < nf; ++i) maxd = dg[i] > maxd ? dg[i] : maxd;
  const float shift = shift_factor * maxd;
  double rr = 0.0, nf2 = 0.0;
  for (long long i = 0; i < nf; ++i) {
    r[i] = f[S.free_idx[i]];
    nf2 += (double)r[i] * r[i];
    if (dg[i] <= shift) dg[i] = shift;
    z[i] = r[i] / dg[i];
    p[i] = z[i];
  }
  const float norm_f = (float)sqrt(nf2);
  float rz_old = 0.0f;
  for (long long i = 0; i < nf; ++i) rz_old += r[i] * z[i];
  int it = 0;
  double res = 0.0;
  if (norm_f == 0.0f) {
    *relres = 0.0;
    *iters_done = 0;
  } else {
    for (it = 1; it <= max_iter; ++it) {
      cpu_apply(&S, p, Ap);
      float pAp = 0.0f;
      for (long long i = 0; i < nf; ++i) {
        Ap[i] += shift * p[i];
        pAp += p[i] * Ap[i];
      }
      const float alpha = rz_old / pAp;
      rr = 0.0;
      float rrf = 0.0f;
      for (long long i = 0; i < nf; ++i) {
        x[i] += alpha * p[i];
        r[i] -= alpha * Ap[i];
        rrf += r[i] * r[i];
      }
      res = sqrt((double)rrf) / norm_f;
      if (res < tol) break;
      float rz_new = 0.0f;
      for (long long i = 0; i < nf; ++i) {
        z[i] = r[i] / dg[i];
        rz_new += r[i] * z[i];
      }
      const float beta = rz_new / rz_old;
      for (long long i = 0; i < nf; ++i) p[i] = z[i] + beta * p[i];
      rz_old = rz_new;
      if (max_seconds > 0 && now_s() - t0 > max_seconds) break;
    }
    if (it > max_iter) it = max_iter;
    *relres = res;
    *iters_done = it;
  }
  *seconds = now_s() - t0;
  memset(x_out, 0, sizeof(float) * S.ndof);
  for (long long i = 0; i < nf; ++i) x_out[S.free_idx[i]] = x[i];
  free(S.free_idx); free(S.partial); free(S.xfull); free(S.yfull);
  free(x); free(r); free(z); free(p); free(Ap); free(dg);
  (void)rr;
  return *iters_done;
}

int ho_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
