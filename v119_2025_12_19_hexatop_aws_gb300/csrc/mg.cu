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
    // children past the fine grid (a coarse axis rounded up from an odd one) count as void
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int a = 0; a < 2; ++a)
          if (2 * I + a < gf.nx && 2 * J + b < gf.ny && 2 * K + c < gf.nz)
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
__device__ __forceinline__ void restrict_node(const Grid& gf, const T* __restrict__ rf, const Grid& gc, const Mask& mc,
                                              T* __restrict__ bc, int I, int J, int K) {
  {
    const long long n = (long long)I + (long long)gc.NX * ((long long)J + (long long)gc.NY * K);
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
__device__ __forceinline__ void restrict_body(const Grid& gf, const T* __restrict__ rf, const Grid& gc, const Mask& mc,
                                              T* __restrict__ bc, long long first, long long stride) {
  const long long nn = gc.nnode();
  for (long long n = first; n < nn; n += stride) {
    const int I = (int)(n % gc.NX);
    const long long t = n / gc.NX;
    restrict_node<T>(gf, rf, gc, mc, bc, I, (int)(t % gc.NY), (int)(t / gc.NY));
  }
}
// Single-grid launches index nodes in 3D (block (32, 4), grid (x, y, z) over
// (I, J, K)): no integer division per node.  With ncol columns (vectors ndof
// apart) grid z runs over K and the column: blockIdx.z = K + NZ * column.
static inline dim3 node_grid3(const Grid& g, int ncol = 1) {
  return dim3((unsigned)((g.NX + 31) / 32), (unsigned)((g.NY + 3) / 4), (unsigned)(g.NZ * ncol));
}
// Columns per launch so that grid z = NZ * columns stays within 65535.
static inline int cols_per_launch(const Grid& g) { return std::max(1, 65535 / g.NZ); }
template <typename T>
__global__ void restrict_kernel(Grid gf, const T* __restrict__ rf, Grid gc, Mask mc, T* __restrict__ bc,
                                const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  const int K = blockIdx.z % gc.NZ, col = blockIdx.z / gc.NZ;
  const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 4 + threadIdx.y;
  if (I < gc.NX && J < gc.NY)
    restrict_node<T>(gf, rf + (long long)col * gf.ndof(), gc, mc, bc + (long long)col * gc.ndof(), I, J, K);
}
template <typename T>
int launch_restrict(const Grid& gf, const T* rf, const Grid& gc, const Mask& mc, T* bc, const int* halt,
                    cudaStream_t st, int ncol) {
  const int per = cols_per_launch(gc);
  int n = 0;
  for (int c0 = 0; c0 < ncol; c0 += per, ++n)
    restrict_kernel<T><<<node_grid3(gc, std::min(per, ncol - c0)), dim3(32, 4), 0, st>>>(
        gf, rf + (long long)c0 * gf.ndof(), gc, mc, bc + (long long)c0 * gc.ndof(), halt);
  return n;
}

// x_f += P x_c.  One thread per coarse node (I, J, K) adds the correction to
// the up-to-8 fine nodes (2I + a, 2J + b, 2K + c), a, b, c in {0, 1}, from
// the coarse corner values (I..I+a, J..J+b, K..K+c) it loads once: fine node
// (a, b, c) gets w = 2^-(a+b+c) times their sum taken in (c, b, a) order.
// Fixed fine DOFs are left alone.  All loads of the thread are issued before
// its arithmetic (loading each fine value next to its update made the mixed
// solve on the 384x192x192 grid 2.5 % slower).
template <typename T>
__device__ __forceinline__ void prolong_add_cnode(const Grid& gc, const T* __restrict__ xc, const Grid& gf,
                                                  const Mask& mf, T* __restrict__ xf, int I, int J, int K) {
  T X[2][2][2][3];
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const bool in = I + a < gc.NX && J + b < gc.NY && K + c < gc.NZ;
        const long long N = (long long)(I + a) + (long long)gc.NX * ((long long)(J + b) + (long long)gc.NY * (K + c));
#pragma unroll
        for (int q = 0; q < 3; ++q) X[c][b][a][q] = in ? xc[3 * N + q] : T(0);
      }
  T Fv[2][2][2][3];
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int i = 2 * I + a, j = 2 * J + b, k = 2 * K + c;
        const bool in = i < gf.NX && j < gf.NY && k < gf.NZ;
        const long long n = (long long)i + (long long)gf.NX * ((long long)j + (long long)gf.NY * k);
#pragma unroll
        for (int q = 0; q < 3; ++q) Fv[c][b][a][q] = in ? xf[3 * n + q] : T(0);
      }
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int k = 2 * K + c;
    if (k >= gf.NZ) continue;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int j = 2 * J + b;
      if (j >= gf.NY) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int i = 2 * I + a;
        if (i >= gf.NX) continue;
        const long long n = (long long)i + (long long)gf.NX * ((long long)j + (long long)gf.NY * k);
        const unsigned fx = fixed_bits(gf, mf, i, j, k, n);
        if (fx == 7u) continue;
        const T w = (a ? T(0.5) : T(1)) * (b ? T(0.5) : T(1)) * (c ? T(0.5) : T(1));
        T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
        for (int cc = 0; cc <= c; ++cc)
#pragma unroll
          for (int bb = 0; bb <= b; ++bb)
#pragma unroll
            for (int aa = 0; aa <= a; ++aa) {
              s0 += X[cc][bb][aa][0];
              s1 += X[cc][bb][aa][1];
              s2 += X[cc][bb][aa][2];
            }
        if (!(fx & 1u)) xf[3 * n] = Fv[c][b][a][0] + w * s0;
        if (!(fx & 2u)) xf[3 * n + 1] = Fv[c][b][a][1] + w * s1;
        if (!(fx & 4u)) xf[3 * n + 2] = Fv[c][b][a][2] + w * s2;
      }
    }
  }
}
template <typename T>
__global__ void prolong_add_kernel(Grid gc, const T* __restrict__ xc, Grid gf, Mask mf, T* __restrict__ xf,
                                   const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  const int K = blockIdx.z % gc.NZ, col = blockIdx.z / gc.NZ;
  const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 4 + threadIdx.y;
  if (I >= gc.NX || J >= gc.NY) return;
  prolong_add_cnode<T>(gc, xc + (long long)col * gc.ndof(), gf, mf, xf + (long long)col * gf.ndof(), I, J, K);
}
template <typename T>
int launch_prolong_add(const Grid& gc, const T* xc, const Grid& gf, const Mask& mf, T* xf, const int* halt,
                       cudaStream_t st, int ncol) {
  const int per = cols_per_launch(gc);
  int n = 0;
  for (int c0 = 0; c0 < ncol; c0 += per, ++n)
    prolong_add_kernel<T><<<node_grid3(gc, std::min(per, ncol - c0)), dim3(32, 4), 0, st>>>(
        gc, xc + (long long)c0 * gc.ndof(), gf, mf, xf + (long long)c0 * gf.ndof(), halt);
  return n;
}

template <typename T>
__device__ __forceinline__ void jacobi0_node(const Grid& g, const Mask& m, const T* __restrict__ fac,
                                             const ModalK<T>& K, int quirk, T sigma, T omega,
                                             const T* __restrict__ b, T* __restrict__ x, int i, int j, int k) {
  {
    const long long n = (long long)i + (long long)g.NX * ((long long)j + (long long)g.NY * k);
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
__device__ __forceinline__ void jacobi0_body(const Grid& g, const Mask& m, const T* __restrict__ fac,
                                             const ModalK<T>& K, int quirk, T sigma, T omega,
                                             const T* __restrict__ b, T* __restrict__ x, long long first,
                                             long long stride) {
  const long long nn = g.nnode();
  for (long long n = first; n < nn; n += stride) {
    const int i = (int)(n % g.NX);
    const long long t = n / g.NX;
    jacobi0_node<T>(g, m, fac, K, quirk, sigma, omega, b, x, i, (int)(t % g.NY), (int)(t / g.NY));
  }
}
// Single grid: a thread takes kJ0Z nodes of its (i, j) column in z, loads
// the factors of the kJ0Z + 1 element layers around them (4 per layer) and
// their b values before any arithmetic, and carries the factor sum of the 4
// elements below a node from the node before (each node needs 4 new factors
// instead of 8).  The diagonal's factor sum is built in jacobi0_node's order
// (the 4 elements below, then the 4 above, each (dy, dx) in turn; an element
// off the grid adds +0, which leaves the sum's bits unchanged).
constexpr int kJ0Z = 4;
template <typename T>
__global__ void jacobi0_kernel(Grid g, Mask m, const T* __restrict__ fac, ModalK<T> K, int quirk, T sigma,
                               T omega, const T* __restrict__ b, T* __restrict__ x, const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  const int nzc = (g.NZ + kJ0Z - 1) / kJ0Z;
  const int zc = blockIdx.z % nzc, col = blockIdx.z / nzc;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 4 + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const long long co = (long long)col * g.ndof();
  b += co;
  x += co;
  // element (i + dx, j + dy) of layer ek, dx, dy in {-1, 0}, in the order (dy, dx)
  const bool xl = i >= 1, xr = i < g.nx, yl = j >= 1, yr = j < g.ny;
  const int k0 = zc * kJ0Z;
  T fl[kJ0Z + 1][4];
#pragma unroll
  for (int q = 0; q <= kJ0Z; ++q) {
    const int ek = k0 - 1 + q;
    const bool zin = ek >= 0 && ek < g.nz;
    const long long row = (long long)g.nx * ((long long)(j - 1) + (long long)g.ny * ek);
    fl[q][0] = (zin && yl && xl) ? fac[row + i - 1] : T(0);
    fl[q][1] = (zin && yl && xr) ? fac[row + i] : T(0);
    fl[q][2] = (zin && yr && xl) ? fac[row + g.nx + i - 1] : T(0);
    fl[q][3] = (zin && yr && xr) ? fac[row + g.nx + i] : T(0);
  }
  T bv[kJ0Z][3];
#pragma unroll
  for (int q = 0; q < kJ0Z; ++q) {
    const int k = k0 + q;
    const long long n = (long long)i + (long long)g.NX * ((long long)j + (long long)g.NY * k);
#pragma unroll
    for (int c = 0; c < 3; ++c) bv[q][c] = k < g.NZ ? b[3 * n + c] : T(0);
  }
  T below = T(0);
#pragma unroll
  for (int t = 0; t < 4; ++t) below += fl[0][t];
#pragma unroll
  for (int q = 0; q < kJ0Z; ++q) {
    const int k = k0 + q;
    if (k >= g.NZ) break;
    T fs = below, nb = T(0);
#pragma unroll
    for (int t = 0; t < 4; ++t) fs += fl[q + 1][t], nb += fl[q + 1][t];
    below = nb;
    const long long n = (long long)i + (long long)g.NX * ((long long)j + (long long)g.NY * k);
    const unsigned fx = fixed_bits(g, m, i, j, k, n);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T d = fma(K.dd[quirk ? 0 : c], fs, sigma);
      x[3 * n + c] = ((fx >> c) & 1u) ? T(0) : omega * bv[q][c] / d;
    }
  }
}
template <typename T>
int launch_jacobi0(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, int quirk, T sigma, T omega,
                   const T* b, T* x, const int* halt, cudaStream_t st, int ncol) {
  const int nzc = (g.NZ + kJ0Z - 1) / kJ0Z;
  const int per = std::max(1, 65535 / nzc);
  int n = 0;
  for (int c0 = 0; c0 < ncol; c0 += per, ++n) {
    const long long co = (long long)c0 * g.ndof();
    const dim3 grid((unsigned)((g.NX + 31) / 32), (unsigned)((g.NY + 3) / 4), (unsigned)(nzc * std::min(per, ncol - c0)));
    jacobi0_kernel<T><<<grid, dim3(32, 4), 0, st>>>(g, m, fac, K, quirk, sigma, omega, b + co, x + co, halt);
  }
  return n;
}

// ---------------------------------------------------------------------------
// Coarsest-level solve in one launch: a single CTA runs `iters` Jacobi-PCG
// iterations on a small grid (element products into a scratch array, then a
// node gather), with block reductions in a fixed order.  Replaces the
// 3 launches per iteration of the general path when the coarse grid is small.
template <typename T>
__device__ __forceinline__ double cta_sum(double v, double* red) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; ++w) t += red[w];  // every thread sums in the same order
  return t;
}

// CTA sum in the accumulation type A (the FP32 coarse solves sum in FP32:
// FP64 arithmetic runs at a small fraction of the FP32 rate on this part);
// every thread returns the same value, summed in the same order.
template <typename A>
__device__ __forceinline__ A cta_sum_acc(A v, A* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  A t = A(0);
  const int nw = blockDim.x >> 5;
  for (int w = 0; w < nw; ++w) t += red[w];
  return t;
}

__device__ __forceinline__ bool modal_nz_mg(int q, int c, int c2) {
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

// One element's f K0 u_e in the Hadamard basis: corner values h (corner order
// dx + 2dy + 4dz) in, corner contributions wh out.
template <typename T>
__device__ __forceinline__ void coarse_element_product(const ModalK<T>& K, T f, T (&h)[8][3], T (&wh)[8][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int sft = 1 << d;
      T tmp[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) {
        const int lo = cc & ~sft;
        tmp[cc] = (cc & sft) ? (h[lo | sft][c] - h[lo][c]) : (h[lo][c] + h[lo | sft][c]);
      }
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) h[cc][c] = tmp[cc];
    }
#pragma unroll
  for (int mm = 0; mm < 8; ++mm)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int qq = mm ^ (1 << c);
      T s = T(0);
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        if (modal_nz_mg(qq, c, c2)) s = fma(K.B[qq][c][c2], h[qq ^ (1 << c2)][c2], s);
      wh[mm][c] = s * f;
    }
  // inverse transform (the forward butterflies transposed)
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int d = 2; d >= 0; --d) {
      const int sft = 1 << d;
      T tmp[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) {
        const int lo = cc & ~sft;
        tmp[cc] = (cc & sft) ? (wh[lo][c] + wh[lo | sft][c]) : (wh[lo][c] - wh[lo | sft][c]);
      }
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) wh[cc][c] = tmp[cc];
    }
}

template <typename T>
__device__ __forceinline__ void coarse_pcg_body(const Grid& g, const Mask& m, const T* __restrict__ fac,
                                                const ModalK<T>& K, T sigma, const T* __restrict__ dinv,
                                                const T* __restrict__ b, T* x, T* r, T* z, T* p, T* q, T* w,
                                                int iters) {
  __shared__ double red[32];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long long n3 = g.ndof(), ne = g.nelem(), nn = g.nnode();
  double part = 0.0;
  for (long long i = tid; i < n3; i += nthr) {
    const T ri = b[i], zi = dinv[i] * ri;
    x[i] = T(0);
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    part += (double)ri * (double)zi;
  }
  double rz = cta_sum<T>(part, red);
  for (int it = 0; it < iters; ++it) {
    // element products w_e = f_e K0 p_e (Hadamard basis), corner order dx + 2dy + 4dz
    for (long long e = tid; e < ne; e += nthr) {
      const int i = (int)(e % g.nx);
      const long long t = e / g.nx;
      const int j = (int)(t % g.ny), k = (int)(t / g.ny);
      T h[8][3];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) {
        const long long nd = (long long)(i + (cc & 1)) + (long long)g.NX * ((long long)(j + ((cc >> 1) & 1)) + (long long)g.NY * (k + (cc >> 2)));
#pragma unroll
        for (int c = 0; c < 3; ++c) h[cc][c] = p[3 * nd + c];
      }
      T wh[8][3];
      coarse_element_product<T>(K, fac[e], h, wh);
#pragma unroll
      for (int cc = 0; cc < 8; ++cc)
#pragma unroll
        for (int c = 0; c < 3; ++c) w[e * 24 + 3 * cc + c] = wh[cc][c];
    }
    __syncthreads();
    part = 0.0;
    for (long long nd = tid; nd < nn; nd += nthr) {
      const int i = (int)(nd % g.NX);
      const long long t = nd / g.NX;
      const int j = (int)(t % g.NY), k = (int)(t / g.NY);
      const unsigned fx = fixed_bits(g, m, i, j, k, nd);
      T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
      for (int oz = 0; oz < 2; ++oz)
#pragma unroll
        for (int oy = 0; oy < 2; ++oy)
#pragma unroll
          for (int ox = 0; ox < 2; ++ox) {
            const int ei = i - 1 + ox, ej = j - 1 + oy, ek = k - 1 + oz;
            if (ei < 0 || ei >= g.nx || ej < 0 || ej >= g.ny || ek < 0 || ek >= g.nz) continue;
            const long long e = (long long)ei + (long long)g.nx * ((long long)ej + (long long)g.ny * ek);
            const int ln = (1 - ox) + 2 * (1 - oy) + 4 * (1 - oz);
            s0 += w[e * 24 + 3 * ln];
            s1 += w[e * 24 + 3 * ln + 1];
            s2 += w[e * 24 + 3 * ln + 2];
          }
      const T sv[3] = {s0, s1, s2};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T pv = p[3 * nd + c];
        const T qv = ((fx >> c) & 1u) ? T(0) : fma(sigma, pv, sv[c]);
        q[3 * nd + c] = qv;
        part += (double)pv * (double)qv;
      }
    }
    const double pAp = cta_sum<T>(part, red);
    if (!(pAp > 0.0)) break;  // converged to rounding or no curvature left
    const T alpha = (T)(rz / pAp);
    part = 0.0;
    for (long long i = tid; i < n3; i += nthr) {
      x[i] = fma(alpha, p[i], x[i]);
      const T ri = fma(-alpha, q[i], r[i]);
      r[i] = ri;
      const T zi = dinv[i] * ri;
      z[i] = zi;
      part += (double)ri * (double)zi;
    }
    const double rz_new = cta_sum<T>(part, red);
    const T beta = (T)(rz != 0.0 ? rz_new / rz : 0.0);
    rz = rz_new;
    for (long long i = tid; i < n3; i += nthr) p[i] = fma(beta, p[i], z[i]);
    __syncthreads();
  }
}
template <typename T>
__global__ void __launch_bounds__(1024) coarse_pcg_kernel(Grid g, Mask m, const T* __restrict__ fac, ModalK<T> K,
                                                          T sigma, const T* __restrict__ dinv, const T* __restrict__ b,
                                                          T* x, T* r, T* z, T* p, T* q, T* w, int iters,
                                                          const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  coarse_pcg_body<T>(g, m, fac, K, sigma, dinv, b, x, r, z, p, q, w, iters);
}
template <typename T>
void launch_coarse_pcg(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, T sigma, const T* dinv,
                       const T* b, T* x, T* r, T* z, T* p, T* q, T* w, int iters, const int* halt, cudaStream_t st) {
  coarse_pcg_kernel<T><<<1, 1024, 0, st>>>(g, m, fac, K, sigma, dinv, b, x, r, z, p, q, w, iters, halt);
}

// ------------------------------------------------------------ batch forms
__device__ __forceinline__ const BatchInst& batch_inst_vec(const BatchInst* in, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (in[mid].vblk0 <= b) lo = mid;
    else hi = mid - 1;
  }
  return in[lo];
}
__device__ __forceinline__ bool batch_halted(const PcgScalars* s, int id) {
  return s && *((volatile const int*)&s[id].halt);
}

// in[i]: g/m/off = the coarse level, g2/off2 = the fine level; blocks by coarse nodes
template <typename T>
__global__ void batch_restrict_kernel(const BatchInst* in, int ninst, const T* __restrict__ rf, T* __restrict__ bc,
                                      const PcgScalars* s) {
  const BatchInst& I = batch_inst_vec(in, ninst, blockIdx.x);
  if (batch_halted(s, I.id)) return;
  restrict_body<T>(I.g2, rf + I.off2, I.g, I.m, bc + I.off,
                   (long long)(blockIdx.x - I.vblk0) * blockDim.x + threadIdx.x, (long long)I.vnblk * blockDim.x);
}
template <typename T>
void launch_batch_restrict(const BatchInst* in, int ninst, int nblocks, const T* rf, T* bc, const PcgScalars* s,
                           cudaStream_t st) {
  batch_restrict_kernel<T><<<nblocks, 256, 0, st>>>(in, ninst, rf, bc, s);
}

// in[i]: g/m/off = the fine level, g2/off2 = the coarse level; blocks by fine nodes
template <typename T>
__global__ void batch_prolong_add_kernel(const BatchInst* in, int ninst, const T* __restrict__ xc, T* __restrict__ xf,
                                         const PcgScalars* s) {
  const BatchInst& I = batch_inst_vec(in, ninst, blockIdx.x);
  if (batch_halted(s, I.id)) return;
  // the instance's blocks (planned over its fine nodes) stride over its coarse nodes
  const Grid gc = I.g2;
  const long long nn = gc.nnode();
  for (long long N = (long long)(blockIdx.x - I.vblk0) * blockDim.x + threadIdx.x; N < nn;
       N += (long long)I.vnblk * blockDim.x) {
    const int Ic = (int)(N % gc.NX);
    const long long t = N / gc.NX;
    prolong_add_cnode<T>(gc, xc + I.off2, I.g, I.m, xf + I.off, Ic, (int)(t % gc.NY), (int)(t / gc.NY));
  }
}
template <typename T>
void launch_batch_prolong_add(const BatchInst* in, int ninst, int nblocks, const T* xc, T* xf,
                              const PcgScalars* s, cudaStream_t st) {
  batch_prolong_add_kernel<T><<<nblocks, 256, 0, st>>>(in, ninst, xc, xf, s);
}

template <typename T>
__global__ void batch_jacobi0_kernel(const BatchInst* in, int ninst, const T* __restrict__ fac, ModalK<T> K, int quirk,
                                     T omega, const T* __restrict__ b, T* __restrict__ x, const PcgScalars* s) {
  const BatchInst& I = batch_inst_vec(in, ninst, blockIdx.x);
  if (batch_halted(s, I.id)) return;
  jacobi0_body<T>(I.g, I.m, fac + I.eoff, K, quirk, (T)I.sigma, omega, b + I.off, x + I.off,
                  (long long)(blockIdx.x - I.vblk0) * blockDim.x + threadIdx.x, (long long)I.vnblk * blockDim.x);
}
template <typename T>
void launch_batch_jacobi0(const BatchInst* in, int ninst, int nblocks, const T* fac, const ModalK<T>& K, int quirk,
                          T omega, const T* b, T* x, const PcgScalars* s, cudaStream_t st) {
  batch_jacobi0_kernel<T><<<nblocks, 256, 0, st>>>(in, ninst, fac, K, quirk, omega, b, x, s);
}

// CTA i solves instance in[i] (vectors at off, element scratch w at 24 * eoff)
template <typename T>
__global__ void __launch_bounds__(1024) batch_coarse_pcg_kernel(const BatchInst* in, const T* __restrict__ fac,
                                                                ModalK<T> K, const T* __restrict__ dinv,
                                                                const T* __restrict__ b, T* x, T* r, T* z, T* p, T* q,
                                                                T* w, int iters, const PcgScalars* s) {
  const BatchInst& I = in[blockIdx.x];
  if (batch_halted(s, I.id)) return;
  const long long o = I.off;
  coarse_pcg_body<T>(I.g, I.m, fac + I.eoff, K, (T)I.sigma, dinv + o, b + o, x + o, r + o, z + o, p + o, q + o,
                     w + 24 * I.eoff, iters);
}
// The same Jacobi-PCG of one instance's coarsest grid with its five vectors
// (x, r, z, p, q) and element factors held in shared memory, so every pass of
// an iteration reads and writes shared memory instead of global memory.  Two
// forms of the product q = A p:
//  * W (scratch): every element's 24 products go to a shared scratch (entry
//    (corner cc, component c) of element e at [(3 cc + c) nElem + e]), then
//    each node sums its up-to-8 entries in a fixed order: one pass over the
//    elements, one over the nodes, 4 barriers per iteration;
//  * colour: the products are added into q in 8 colour passes (elements of
//    one parity in x, y and z share no node), so no scratch is needed, at 8
//    barriers more per iteration.
// Both sum in a fixed order and in T (FP32 sums: FP64 arithmetic runs at a
// small fraction of the FP32 rate on this part).  One CTA per instance, x
// written to xout at the end.
template <typename T, bool W>
__global__ void __launch_bounds__(1024) batch_coarse_pcg_smem_kernel(const BatchInst* in, const T* __restrict__ fac,
                                                                     ModalK<T> K, const T* __restrict__ dinv,
                                                                     const T* __restrict__ b, T* xout, int iters,
                                                                     const PcgScalars* s) {
  extern __shared__ __align__(16) unsigned char coarse_smem[];
  __shared__ T red[32];
  const BatchInst& I = in[blockIdx.x];
  if (batch_halted(s, I.id)) return;
  const Grid g = I.g;
  const Mask m = I.m;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int n3 = (int)g.ndof(), ne = (int)g.nelem(), nn = (int)g.nnode();
  T* sx = (T*)coarse_smem;
  T* sr = sx + n3;
  T* sz = sr + n3;
  T* sp = sz + n3;
  T* sq = sp + n3;
  T* sf = sq + n3;
  T* sw = sf + ne;  // W form only: 24 nElem words
  const T* gb = b + I.off;
  const T* gd = dinv + I.off;
  const T* gf = fac + I.eoff;
  T part = T(0);
  for (int e = tid; e < ne; e += nthr) sf[e] = gf[e];
  for (int i = tid; i < n3; i += nthr) {
    const T ri = gb[i], zi = gd[i] * ri;
    sx[i] = T(0);
    sr[i] = ri;
    sz[i] = zi;
    sp[i] = zi;
    part = fma(ri, zi, part);
  }
  T rz = cta_sum_acc<T>(part, red);
  const T sigma = (T)I.sigma;
  for (int it = 0; it < iters; ++it) {
    if constexpr (W) {
      for (int e = tid; e < ne; e += nthr) {
        const int i = e % g.nx, t = e / g.nx, j = t % g.ny, k = t / g.ny;
        T h[8][3];
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const int nd = (i + (cc & 1)) + g.NX * ((j + ((cc >> 1) & 1)) + g.NY * (k + (cc >> 2)));
#pragma unroll
          for (int c = 0; c < 3; ++c) h[cc][c] = sp[3 * nd + c];
        }
        T wh[8][3];
        coarse_element_product<T>(K, sf[e], h, wh);
#pragma unroll
        for (int cc = 0; cc < 8; ++cc)
#pragma unroll
          for (int c = 0; c < 3; ++c) sw[(3 * cc + c) * ne + e] = wh[cc][c];
      }
      __syncthreads();
    } else {
      for (int i = tid; i < n3; i += nthr) sq[i] = T(0);
      __syncthreads();
      for (int color = 0; color < 8; ++color) {
        const int cx = color & 1, cy = (color >> 1) & 1, cz = color >> 2;
        const int mx = (g.nx - cx + 1) >> 1, my = (g.ny - cy + 1) >> 1, mz = (g.nz - cz + 1) >> 1;
        const int mc = mx * my * mz;
        for (int t = tid; t < mc; t += nthr) {
          const int i = 2 * (t % mx) + cx, j = 2 * ((t / mx) % my) + cy, k = 2 * (t / (mx * my)) + cz;
          T h[8][3];
#pragma unroll
          for (int cc = 0; cc < 8; ++cc) {
            const int nd = (i + (cc & 1)) + g.NX * ((j + ((cc >> 1) & 1)) + g.NY * (k + (cc >> 2)));
#pragma unroll
            for (int c = 0; c < 3; ++c) h[cc][c] = sp[3 * nd + c];
          }
          T wh[8][3];
          coarse_element_product<T>(K, sf[i + g.nx * (j + g.ny * k)], h, wh);
#pragma unroll
          for (int cc = 0; cc < 8; ++cc) {
            const int nd = (i + (cc & 1)) + g.NX * ((j + ((cc >> 1) & 1)) + g.NY * (k + (cc >> 2)));
#pragma unroll
            for (int c = 0; c < 3; ++c) sq[3 * nd + c] += wh[cc][c];
          }
        }
        __syncthreads();
      }
    }
    part = T(0);
    for (int nd = tid; nd < nn; nd += nthr) {
      const int i = nd % g.NX, t = nd / g.NX, j = t % g.NY, k = t / g.NY;
      const unsigned fx = fixed_bits(g, m, i, j, k, nd);
      T sv[3];
      if constexpr (W) {
        sv[0] = sv[1] = sv[2] = T(0);
#pragma unroll
        for (int oz = 0; oz < 2; ++oz)
#pragma unroll
          for (int oy = 0; oy < 2; ++oy)
#pragma unroll
            for (int ox = 0; ox < 2; ++ox) {
              const int ei = i - 1 + ox, ej = j - 1 + oy, ek = k - 1 + oz;
              if (ei < 0 || ei >= g.nx || ej < 0 || ej >= g.ny || ek < 0 || ek >= g.nz) continue;
              const int e = ei + g.nx * (ej + g.ny * ek);
              const int ln = (1 - ox) + 2 * (1 - oy) + 4 * (1 - oz);
#pragma unroll
              for (int c = 0; c < 3; ++c) sv[c] += sw[(3 * ln + c) * ne + e];
            }
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) sv[c] = sq[3 * nd + c];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T pv = sp[3 * nd + c];
        const T qv = ((fx >> c) & 1u) ? T(0) : fma(sigma, pv, sv[c]);
        sq[3 * nd + c] = qv;
        part = fma(pv, qv, part);
      }
    }
    const T pAp = cta_sum_acc<T>(part, red);
    if (!(pAp > T(0))) break;  // converged to rounding or no curvature left
    const T alpha = rz / pAp;
    part = T(0);
    for (int i = tid; i < n3; i += nthr) {
      sx[i] = fma(alpha, sp[i], sx[i]);
      const T ri = fma(-alpha, sq[i], sr[i]);
      sr[i] = ri;
      const T zi = gd[i] * ri;
      sz[i] = zi;
      part = fma(ri, zi, part);
    }
    const T rz_new = cta_sum_acc<T>(part, red);
    const T beta = rz != T(0) ? rz_new / rz : T(0);
    rz = rz_new;
    for (int i = tid; i < n3; i += nthr) sp[i] = fma(beta, sp[i], sz[i]);
    __syncthreads();
  }
  T* gx = xout + I.off;
  for (int i = tid; i < n3; i += nthr) gx[i] = sx[i];
}

// Shared memory a smem form needs for the largest coarsest grid of a launch
// (0: too large for that form).
template <typename T>
size_t batch_coarse_smem_bytes(long long max_ndof, long long max_nelem, bool scratch) {
  const size_t bytes = (size_t)(5 * max_ndof + max_nelem * (scratch ? 25 : 1)) * sizeof(T);
  return bytes <= 220u * 1024u ? bytes : 0;
}

template <typename T>
void launch_batch_coarse_pcg(const BatchInst* in, int ninst, const T* fac, const ModalK<T>& K, const T* dinv,
                             const T* b, T* x, T* r, T* z, T* p, T* q, T* w, int iters, const PcgScalars* s,
                             cudaStream_t st, long long max_ndof, long long max_nelem) {
  const size_t smem_w = batch_coarse_smem_bytes<T>(max_ndof, max_nelem, true);
  const size_t smem_c = batch_coarse_smem_bytes<T>(max_ndof, max_nelem, false);
  static bool attr = false;
  if (!attr && smem_c > 0) {
    cudaFuncSetAttribute(batch_coarse_pcg_smem_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(batch_coarse_pcg_smem_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  if (smem_w > 0) {
    batch_coarse_pcg_smem_kernel<T, true><<<ninst, 1024, smem_w, st>>>(in, fac, K, dinv, b, x, iters, s);
    return;
  }
  if (smem_c > 0) {
    batch_coarse_pcg_smem_kernel<T, false><<<ninst, 1024, smem_c, st>>>(in, fac, K, dinv, b, x, iters, s);
    return;
  }
  batch_coarse_pcg_kernel<T><<<ninst, 1024, 0, st>>>(in, fac, K, dinv, b, x, r, z, p, q, w, iters, s);
}

// Exact coarsest-level solve: x = A^-1 b with the dense symmetric inverse
// (n x n, zero rows/columns at fixed DOFs).  CTA = 32 rows, 8 warps split the
// columns; lane = row, so each column read is one coalesced 128-byte access.
// blockIdx.y picks one of ncol right-hand sides (vectors n apart).
template <typename T>
__global__ void __launch_bounds__(256) dense_coarse_kernel(int n, const T* __restrict__ A, const T* __restrict__ b,
                                                           T* __restrict__ x, const int* halt) {
  if (halt && *((volatile const int*)halt)) return;
  b += (long long)blockIdx.y * n;
  x += (long long)blockIdx.y * n;
  __shared__ T part[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = blockIdx.x * 32 + lane;
  T s = T(0);
  if (row < n)
    for (int j = w; j < n; j += 8) s = fma(A[(long long)j * n + row], b[j], s);
  part[w][lane] = s;
  __syncthreads();
  if (w == 0 && row < n) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < 8; ++q) t += part[q][lane];
    x[row] = t;
  }
}
template <typename T>
void launch_dense_coarse(long long n, const T* A, const T* b, T* x, const int* halt, cudaStream_t st, int ncol) {
  dense_coarse_kernel<T><<<dim3((unsigned)((n + 31) / 32), (unsigned)ncol), 256, 0, st>>>((int)n, A, b, x, halt);
}

#define INST(T)                                                                                     \
  template void launch_coarsen_factors<T>(const Grid&, const T*, const Grid&, T*, cudaStream_t);    \
  template int launch_restrict<T>(const Grid&, const T*, const Grid&, const Mask&, T*, const int*,  \
                                  cudaStream_t, int);                                               \
  template int launch_prolong_add<T>(const Grid&, const T*, const Grid&, const Mask&, T*,           \
                                     const int*, cudaStream_t, int);                                \
  template int launch_jacobi0<T>(const Grid&, const Mask&, const T*, const ModalK<T>&, int, T, T,   \
                                 const T*, T*, const int*, cudaStream_t, int);                      \
  template void launch_coarse_pcg<T>(const Grid&, const Mask&, const T*, const ModalK<T>&, T, const T*, \
                                     const T*, T*, T*, T*, T*, T*, T*, int, const int*, cudaStream_t);     \
  template void launch_dense_coarse<T>(long long, const T*, const T*, T*, const int*, cudaStream_t, int); \
  template void launch_batch_restrict<T>(const BatchInst*, int, int, const T*, T*, const PcgScalars*,     \
                                         cudaStream_t);                                                   \
  template void launch_batch_prolong_add<T>(const BatchInst*, int, int, const T*, T*, const PcgScalars*,  \
                                            cudaStream_t);                                                \
  template void launch_batch_jacobi0<T>(const BatchInst*, int, int, const T*, const ModalK<T>&, int, T,   \
                                        const T*, T*, const PcgScalars*, cudaStream_t);                   \
  template void launch_batch_coarse_pcg<T>(const BatchInst*, int, const T*, const ModalK<T>&, const T*,   \
                                           const T*, T*, T*, T*, T*, T*, T*, int, const PcgScalars*,      \
                                           cudaStream_t, long long, long long);
INST(double)
INST(float)
#undef INST

}  // namespace hexa
