// (e) SIMP strain-energy sensitivities and the optimality-criteria update.
//
// The reference has neither (its modulus is linear in density,
// src/Solvers/GPUSolver.jl:254, and its update is a stress-ratio rule,
// src/Optimization/TopOpt.jl:211-482).  These kernels restate the published
// SIMP / OC method (Bendsoe & Sigmund; the OC update of Andreassen et al.
// 2011, "Efficient topology optimization in MATLAB using 88 lines of code"):
//   E_e  = Emin + rho_e^p (E0 - Emin)
//   ce_e = u_e^T K0 u_e           (K0 for E = 1)
//   c    = sum_e E_e ce_e,  dc_e = -p rho_e^(p-1) (E0 - Emin) ce_e
//   x_new = clamp(x * sqrt(-dc / (lambda dv)), max(0, x-move), min(1, x+move))
// with lambda found by bisection so that mean(x_new) = volfrac.  The element
// energy uses the same Hadamard-basis blocks as the operator: ce = u_hat^T B u_hat.
#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

static inline int topo_blocks(long long n) {
  long long b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 8) b = 152 * 8;
  return (int)b;
}

__global__ void simp_factors_kernel(const double* __restrict__ rho, double Emin, double E0, double penal,
                                    double* __restrict__ fac, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    fac[e] = Emin + pow(rho[e], penal) * (E0 - Emin);
}
void launch_simp_factors(const double* rho, double Emin, double E0, double penal, double* fac, long long n,
                         cudaStream_t st) {
  simp_factors_kernel<<<topo_blocks(n), 256, 0, st>>>(rho, Emin, E0, penal, fac, n);
}

__device__ __forceinline__ bool modal_nz_dev(int q, int c, int c2) {
  if (q == 1 || q == 2 || q == 4) {
    const int c0 = (q == 1) ? 0 : (q == 2 ? 1 : 2);
    return c != c0 && c2 != c0;
  }
  if (q == 3 || q == 5 || q == 6) {
    const int cf = (q == 3) ? 2 : (q == 5 ? 1 : 0);
    return (c == cf) == (c2 == cf);
  }
  return true;
}

__global__ void sens_kernel(Grid g, ModalK<double> K, const double* __restrict__ rho, const double* __restrict__ u,
                            double Emin, double E0, double penal, double* __restrict__ dc, RedArgs red) {
  double acc[1] = {0.0};
  const long long ne = g.nelem();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.nx);
    const long long t = e / g.nx;
    const int j = (int)(t % g.ny), k = (int)(t / g.ny);
    double v[8][3];
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {
      const long long n = (long long)(i + (cc & 1)) + (long long)g.NX * ((long long)(j + ((cc >> 1) & 1)) + (long long)g.NY * (k + (cc >> 2)));
#pragma unroll
      for (int c = 0; c < 3; ++c) v[cc][c] = __ldg(u + 3 * n + c);
    }
    // 3-D Hadamard transform per component: modes m = mx + 2my + 4mz
    double h[8][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double a[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) a[cc] = v[cc][c];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int s = 1 << d;
        double b2[8];
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const int lo = cc & ~s;
          b2[cc] = (cc & s) ? (a[lo | s] - a[lo]) : (a[lo] + a[lo | s]);
        }
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) a[cc] = b2[cc];
      }
#pragma unroll
      for (int m = 0; m < 8; ++m) h[m][c] = a[m];
    }
    double ce = 0.0;
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int q = m ^ (1 << c);
        double w = 0.0;
#pragma unroll
        for (int c2 = 0; c2 < 3; ++c2)
          if (modal_nz_dev(q, c, c2)) w = fma(K.B[q][c][c2], h[q ^ (1 << c2)][c2], w);
        ce = fma(h[m][c], w, ce);
      }
    const double r = rho[e];
    const double rp1 = pow(r, penal - 1.0);
    dc[e] = -penal * rp1 * (E0 - Emin) * ce;
    acc[0] += (Emin + rp1 * r * (E0 - Emin)) * ce;
  }
  block_reduce_finalize<1>(red, acc);
}
void launch_sensitivities(const Grid& g, const ModalK<double>& K, const double* rho, const double* u, double Emin,
                          double E0, double penal, double* dc, const RedArgs& red, cudaStream_t st) {
  sens_kernel<<<topo_blocks(g.nelem()), 256, 0, st>>>(g, K, rho, u, Emin, E0, penal, dc, red);
}

__device__ __forceinline__ double oc_new(double x, double dc, double dv, double lam, double move) {
  const double be = x * sqrt(-dc / dv / lam);
  return fmax(0.0, fmax(x - move, fmin(1.0, fmin(x + move, be))));
}

// Sum over elements of x_new(lambda_q) for nlam candidate multipliers; block
// partials [block][nlam] are summed in block order by the caller's finalize.
__global__ void oc_volumes_kernel(const double* __restrict__ x, const double* __restrict__ dc,
                                  const double* __restrict__ dv, long long n, const double* __restrict__ lam, int nlam,
                                  double move, double* __restrict__ partials) {
  __shared__ double sl[32];
  __shared__ double sw[8][32];
  if (threadIdx.x < nlam) sl[threadIdx.x] = lam[threadIdx.x];
  __syncthreads();
  double acc[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) acc[q] = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double xe = x[e], de = dc[e], ve = dv[e];
#pragma unroll
    for (int q = 0; q < 32; ++q)
      if (q < nlam) acc[q] += oc_new(xe, de, ve, sl[q], move);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 32; ++q) {
    double t = warp_sum(acc[q]);
    if (lane == q) sw[wid][q] = t;
  }
  __syncthreads();
  if (threadIdx.x < nlam) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sw[w][threadIdx.x];
    partials[(long long)blockIdx.x * 32 + threadIdx.x] = t;
  }
}
void launch_oc_volumes(const double* x, const double* dc, const double* dv, long long n, const double* lam, int nlam,
                       double move, double* partials, int nblocks, cudaStream_t st) {
  oc_volumes_kernel<<<nblocks, 256, 0, st>>>(x, dc, dv, n, lam, nlam, move, partials);
}

__global__ void oc_apply_kernel(const double* __restrict__ x, const double* __restrict__ dc, const double* __restrict__ dv,
                                long long n, double lam, double move, double* __restrict__ xout) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    xout[e] = oc_new(x[e], dc[e], dv[e], lam, move);
}
void launch_oc_apply(const double* x, const double* dc, const double* dv, long long n, double lam, double move,
                     double* xout, cudaStream_t st) {
  oc_apply_kernel<<<topo_blocks(n), 256, 0, st>>>(x, dc, dv, n, lam, move, xout);
}

}  // namespace hexa
