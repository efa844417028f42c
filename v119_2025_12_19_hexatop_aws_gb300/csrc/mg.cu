// (c) Geometric multigrid transfer and smoothing kernels.
//
// The reference's "multigrid" (src/Solvers/GPUGeometricMultigrid.jl:57-346)
// is a two-level additive preconditioner whose restriction scatters with
// 8x3 Float32 atomics per fine node (:57-138) from normalised coordinates,
// and whose coarse operator is only a diagonal.  Here the hierarchy is a real
// V-cycle on nested 2:1 grids: restriction is the exact transpose of the
// trilinear prolongation in gather form (27 fine nodes per coarse node, no
// atomics), prolongation is fused with the correction add, coarse operators
// are rediscretised (K0 at 2h = 2 K0(h), factor = mean of the 8 children),
// and the first damped-Jacobi sweep from a zero guess is a pointwise pass.
#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

static inline int mg_blocks(long long n, int threads = 256) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (int)b;
}

template <typename T>
__global__ void coarsen_factors_kernel(Grid gf, const T* __restrict__ ff, Grid gc, T* __restrict__ fc) {
  const long long ne = gc.nelem();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne;
       e += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(e % gc.nx);
    const long long t = e / gc.nx;
    const int J = (int)(t % gc.ny), K = (int)(t / gc.ny);
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int a = 0; a < 2; ++a)
          s += ff[(long long)(2 * I + a) + (long long)gf.nx * ((long long)(2 * J + b) + (long long)gf.ny * (2 * K + c))];
    fc[e] = T(0.25) * s;  // 2 * (sum / 8)
  }
}
template <typename T>
void launch_coarsen_factors(const Grid& gf, const T* ff, const Grid& gc, T* fc, cudaStream_t st) {
  coarsen_factors_kernel<T><<<mg_blocks(gc.nelem()), 256, 0, st>>>(gf, ff, gc, fc);
}

__global__ void coarsen_mask_kernel(Grid gf, const uint8_t* __restrict__ mf, Grid gc, uint8_t* __restrict__ mc) {
  const long long nn = gc.nnode();
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(n % gc.NX);
    const long long t = n / gc.NX;
    const int J = (int)(t % gc.NY), K = (int)(t / gc.NY);
    mc[n] = mf[(long long)(2 * I) + (long long)gf.NX * ((long long)(2 * J) + (long long)gf.NY * (2 * K))];
  }
}
void launch_coarsen_mask(const Grid& gf, const uint8_t* mf, const Grid& gc, uint8_t* mc, cudaStream_t st) {
  coarsen_mask_kernel<<<mg_blocks(gc.nnode()), 256, 0, st>>>(gf, mf, gc, mc);
}

template <typename T>
__global__ void restrict_kernel(Grid gf, const T* __restrict__ rf, Grid gc, Mask mc, T* __restrict__ bc,
                                const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  const long long nn = gc.nnode();
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(n % gc.NX);
    const long long t = n / gc.NX;
    const int J = (int)(t % gc.NY), K = (int)(t / gc.NY);
    const unsigned fx = fixed_bits(gc, mc, I, J, K, n);
    T s0 = T(0), s1 = T(0), s2 = T(0);
    if (fx != 7u) {
      for (int dk = -1; dk <= 1; ++dk) {
        const int k = 2 * K + dk;
        if (k < 0 || k >= gf.NZ) continue;
        const T wk = dk ? T(0.5) : T(1);
        for (int dj = -1; dj <= 1; ++dj) {
          const int j = 2 * J + dj;
          if (j < 0 || j >= gf.NY) continue;
          const T wjk = (dj ? T(0.5) : T(1)) * wk;
          const long long row = (long long)gf.NX * ((long long)j + (long long)gf.NY * k);
#pragma unroll
          for (int di = -1; di <= 1; ++di) {
            const int i = 2 * I + di;
            if (i < 0 || i >= gf.NX) continue;
            const T w = (di ? T(0.5) : T(1)) * wjk;
            const long long f = 3 * (row + i);
            s0 = fma(w, rf[f], s0);
            s1 = fma(w, rf[f + 1], s1);
            s2 = fma(w, rf[f + 2], s2);
          }
        }
      }
    }
    bc[3 * n] = (fx & 1u) ? T(0) : s0;
    bc[3 * n + 1] = (fx & 2u) ? T(0) : s1;
    bc[3 * n + 2] = (fx & 4u) ? T(0) : s2;
  }
}
template <typename T>
void launch_restrict(const Grid& gf, const T* rf, const Grid& gc, const Mask& mc, T* bc, const int* halt,
                     cudaStream_t st) {
  restrict_kernel<T><<<mg_blocks(gc.nnode()), 256, 0, st>>>(gf, rf, gc, mc, bc, halt);
}

template <typename T>
__global__ void prolong_add_kernel(Grid gc, const T* __restrict__ xc, Grid gf, Mask mf, T* __restrict__ xf,
                                   const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  const long long nn = gf.nnode();
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % gf.NX);
    const long long t = n / gf.NX;
    const int j = (int)(t % gf.NY), k = (int)(t / gf.NY);
    const unsigned fx = fixed_bits(gf, mf, i, j, k, n);
    if (fx == 7u) continue;
    const int I0 = i >> 1, J0 = j >> 1, K0 = k >> 1;
    const int ni = (i & 1) ? 2 : 1, nj = (j & 1) ? 2 : 1, nk = (k & 1) ? 2 : 1;
    const T wi = (i & 1) ? T(0.5) : T(1), wj = (j & 1) ? T(0.5) : T(1), wk = (k & 1) ? T(0.5) : T(1);
    const T w = wi * wj * wk;
    T s0 = T(0), s1 = T(0), s2 = T(0);
    for (int c = 0; c < nk; ++c)
      for (int b = 0; b < nj; ++b)
        for (int a = 0; a < ni; ++a) {
          const long long N = (long long)(I0 + a) + (long long)gc.NX * ((long long)(J0 + b) + (long long)gc.NY * (K0 + c));
          s0 += xc[3 * N];
          s1 += xc[3 * N + 1];
          s2 += xc[3 * N + 2];
        }
    if (!(fx & 1u)) xf[3 * n] += w * s0;
    if (!(fx & 2u)) xf[3 * n + 1] += w * s1;
    if (!(fx & 4u)) xf[3 * n + 2] += w * s2;
  }
}
template <typename T>
void launch_prolong_add(const Grid& gc, const T* xc, const Grid& gf, const Mask& mf, T* xf, const int* halt,
                        cudaStream_t st) {
  prolong_add_kernel<T><<<mg_blocks(gf.nnode()), 256, 0, st>>>(gc, xc, gf, mf, xf, halt);
}

template <typename T>
__global__ void jacobi0_kernel(Grid g, Mask m, const T* __restrict__ fac, ModalK<T> K, int quirk, T sigma,
                               T omega, const T* __restrict__ b, T* __restrict__ x, const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  const long long nn = g.nnode();
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % g.NX);
    const long long t = n / g.NX;
    const int j = (int)(t % g.NY), k = (int)(t / g.NY);
    const unsigned fx = fixed_bits(g, m, i, j, k, n);
    T fs = T(0);
#pragma unroll
    for (int dz = -1; dz <= 0; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 0; ++dx) {
          const int ei = i + dx, ej = j + dy, ek = k + dz;
          if (ei >= 0 && ei < g.nx && ej >= 0 && ej < g.ny && ek >= 0 && ek < g.nz)
            fs += fac[(long long)ei + (long long)g.nx * ((long long)ej + (long long)g.ny * ek)];
        }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T d = fma(K.dd[quirk ? 0 : c], fs, sigma);
      x[3 * n + c] = ((fx >> c) & 1u) ? T(0) : omega * b[3 * n + c] / d;
    }
  }
}
template <typename T>
void launch_jacobi0(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, int quirk, T sigma, T omega,
                    const T* b, T* x, const int* halt, cudaStream_t st) {
  jacobi0_kernel<T><<<mg_blocks(g.nnode()), 256, 0, st>>>(g, m, fac, K, quirk, sigma, omega, b, x, halt);
}

#define INST(T)                                                                                     \
  template void launch_coarsen_factors<T>(const Grid&, const T*, const Grid&, T*, cudaStream_t);    \
  template void launch_restrict<T>(const Grid&, const T*, const Grid&, const Mask&, T*, const int*, \
                                   cudaStream_t);                                                   \
  template void launch_prolong_add<T>(const Grid&, const T*, const Grid&, const Mask&, T*,          \
                                      const int*, cudaStream_t);                                    \
  template void launch_jacobi0<T>(const Grid&, const Mask&, const T*, const ModalK<T>&, int, T, T,  \
                                  const T*, T*, const int*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace hexa
