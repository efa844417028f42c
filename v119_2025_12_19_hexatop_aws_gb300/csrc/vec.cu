// (b) Fused PCG vector passes and small helpers.
//
// Replaces the reference's separate broadcasts and CUBLAS calls of one PCG
// iteration (src/Solvers/GPUSolver.jl:372-416: the shift broadcast, dot(p,Ap)
// with a host round trip, two axpys, dot(r,r) every 10 iterations, the Jacobi
// kernel :162-168, dot(r,z) and the p update).  Here one pass does
// x += alpha p, r -= alpha Ap, ||r||^2, z = M^-1 r and r.z with warp-shuffle
// block reductions; the coefficients (alpha, beta) and the convergence test
// live in device memory, so no scalar ever returns to the host inside an
// iteration.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <initializer_list>

#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

static inline int vec_blocks(long long n, int threads = 256, int maxb = 152 * 8) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > maxb) b = maxb;
  return (int)b;
}

// Per-thread partial sums run in the vector's precision for kChunk terms and
// are then folded into FP64: FP64 arithmetic per element would make the FP32
// passes FP64-bound on GB300.
constexpr int kChunk = 32;
template <typename T, int NS>
__device__ __forceinline__ void flush_parts(double (&acc)[NS], T (&part)[NS], int& cnt) {
#pragma unroll
  for (int q = 0; q < NS; ++q) {
    acc[q] += (double)part[q];
    part[q] = T(0);
  }
  cnt = 0;
}

// 16-byte vector access of the PCG passes: W elements per load/store.
template <typename T>
struct V16;
template <>
struct V16<float> {
  using V = float4;
  static constexpr int W = 4;
};
template <>
struct V16<double> {
  using V = double2;
  static constexpr int W = 2;
};
template <typename T>
__device__ __forceinline__ void ldv(const T* p, long long i, T (&a)[V16<T>::W]) {
  *reinterpret_cast<typename V16<T>::V*>(a) = reinterpret_cast<const typename V16<T>::V*>(p)[i];
}
template <typename T>
__device__ __forceinline__ void stv(T* p, long long i, const T (&a)[V16<T>::W]) {
  reinterpret_cast<typename V16<T>::V*>(p)[i] = *reinterpret_cast<const typename V16<T>::V*>(a);
}
// Whether the column bases stay 16-byte aligned: all pointers aligned and
// (one column, or a column length that keeps later columns aligned).
template <typename T>
static bool vec_ok(long long n, int ncol, std::initializer_list<const void*> ptrs) {
  for (const void* q : ptrs)
    if (q && (reinterpret_cast<uintptr_t>(q) & 15u)) return false;
  return ncol <= 1 || (n % V16<T>::W) == 0;
}

template <typename T>
__global__ void fill_kernel(T* v, T val, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = val;
}

template <typename T>
void launch_fill(T* v, T val, long long n, cudaStream_t st) {
  fill_kernel<T><<<vec_blocks(n), 256, 0, st>>>(v, val, n);
}

template <typename T>
__global__ void copy_kernel(T* __restrict__ d, const T* __restrict__ s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = s[i];
}
template <typename T>
void launch_copy(T* dst, const T* src, long long n, cudaStream_t st) {
  copy_kernel<T><<<vec_blocks(n), 256, 0, st>>>(dst, src, n);
}

template <typename TD, typename TS>
__global__ void mask_copy_kernel(Grid g, Mask m, TD* __restrict__ d, const TS* __restrict__ s) {
  const long long nn = g.nnode();
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % g.NX);
    const long long t = n / g.NX;
    const int j = (int)(t % g.NY), k = (int)(t / g.NY);
    const unsigned fx = fixed_bits(g, m, i, j, k, n);
#pragma unroll
    for (int c = 0; c < 3; ++c) d[3 * n + c] = ((fx >> c) & 1u) ? TD(0) : (TD)s[3 * n + c];
  }
}
template <typename TD, typename TS>
void launch_mask_copy(const Grid& g, const Mask& m, TD* dst, const TS* src, cudaStream_t st) {
  mask_copy_kernel<TD, TS><<<vec_blocks(g.nnode()), 256, 0, st>>>(g, m, dst, src);
}

// Sum of the factors of the (up to) 8 elements around node (i,j,k).
template <typename T>
__device__ __forceinline__ T node_factor_sum(const Grid& g, const T* __restrict__ fac, int i, int j,
                                             int k) {
  T s = T(0);
#pragma unroll
  for (int dz = -1; dz <= 0; ++dz)
#pragma unroll
    for (int dy = -1; dy <= 0; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 0; ++dx) {
        const int ei = i + dx, ej = j + dy, ek = k + dz;
        if (ei >= 0 && ei < g.nx && ej >= 0 && ej < g.ny && ek >= 0 && ek < g.nz)
          s += __ldg(fac + (long long)ei + (long long)g.nx * ((long long)ej + (long long)g.ny * ek));
      }
  return s;
}

template <typename T>
__global__ void diag_kernel(Grid g, Mask m, const T* __restrict__ fac, ModalK<T> K, int quirk,
                            T sigma, T* __restrict__ diag, T* __restrict__ dinv) {
  const long long nn = g.nnode();
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % g.NX);
    const long long t = n / g.NX;
    const int j = (int)(t % g.NY), k = (int)(t / g.NY);
    const unsigned fx = fixed_bits(g, m, i, j, k, n);
    const T fs = node_factor_sum<T>(g, fac, i, j, k);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const bool fixd = (fx >> c) & 1u;
      const T d = K.dd[quirk ? 0 : c] * fs;
      if (diag) diag[3 * n + c] = fixd ? T(0) : d;
      if (dinv) dinv[3 * n + c] = fixd ? T(0) : T(1) / (d + sigma);
    }
  }
}
template <typename T>
void launch_diag(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, int quirk, T sigma,
                 T* diag, T* dinv, cudaStream_t st) {
  diag_kernel<T><<<vec_blocks(g.nnode()), 256, 0, st>>>(g, m, fac, K, quirk, sigma, diag, dinv);
}

__global__ void max_kernel(const double* __restrict__ v, long long n, RedArgs red) {
  double mx = -INFINITY;
  bool bad = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double t = v[i];
    if (!(t == t) || isinf(t)) bad = true;
    mx = fmax(mx, t);
  }
  // reduce max through the sum machinery: encode as two passes is overkill;
  // use a shared-memory max then the ticketed finalize on the block maxima.
  __shared__ double sm[32];
  __shared__ int sbad;
  __shared__ bool am_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) sbad = 0;
  __syncthreads();
  if (bad) atomicOr(&sbad, 1);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) sm[wid] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = -INFINITY;
    for (int w = 0; w < nw; ++w) t = fmax(t, sm[w]);
    red.partials[2 * blockIdx.x] = t;
    red.partials[2 * blockIdx.x + 1] = sbad ? 1.0 : 0.0;
    __threadfence();
    const unsigned tk = atomicAdd(red.ticket, 1u);
    am_last = (tk == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last && threadIdx.x == 0) {
    __threadfence();
    double t = -INFINITY, b = 0.0;
    for (unsigned q = 0; q < gridDim.x; ++q) {
      t = fmax(t, ((volatile double*)red.partials)[2 * q]);
      b = fmax(b, ((volatile double*)red.partials)[2 * q + 1]);
    }
    red.dst[0] = (b > 0.0) ? NAN : t;
    *red.ticket = 0u;
  }
}
void launch_max(const double* v, long long n, const RedArgs& red, int nblocks, cudaStream_t st) {
  max_kernel<<<nblocks, 256, 0, st>>>(v, n, red);
}

// Column mapping of the batched passes: block b works on column b % ncol as
// block b / ncol of that column's gridDim.x / ncol blocks.
struct ColMap {
  int col;
  long long first, stride;
};
__device__ __forceinline__ ColMap colmap(int ncol) {
  const int nc = ncol > 1 ? ncol : 1;
  ColMap m;
  m.col = (int)(blockIdx.x % nc);
  const long long j = blockIdx.x / nc, nbc = gridDim.x / nc;
  m.first = j * blockDim.x + threadIdx.x;
  m.stride = nbc * blockDim.x;
  return m;
}
static inline int col_blocks(int nblocks, int ncol) {
  const int nc = ncol > 1 ? ncol : 1;
  const int per = std::max(1, nblocks / nc);
  return per * nc;
}

template <typename T, int NS, bool VEC>
__global__ void dot_kernel(const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c,
                           const T* __restrict__ d, long long n, RedArgs red, const int* halt) {
  const ColMap cm = colmap(red.ncol);
  if (halted(halt, cm.col)) return;
  const long long off = (long long)cm.col * n;
  double acc[NS];
  T part[NS];
#pragma unroll
  for (int q = 0; q < NS; ++q) acc[q] = 0.0, part[q] = T(0);
  int cnt = 0;
  long long tail = 0;
  if (VEC) {
    constexpr int W = V16<T>::W;
    const long long nv = n / W;
    tail = nv * W;
    for (long long i = cm.first; i < nv; i += cm.stride) {
      T av[W], bv[W], cv[W], dv[W];
      ldv(a + off, i, av);
      ldv(b + off, i, bv);
      if (NS > 1) ldv(c + off, i, cv), ldv(d + off, i, dv);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        part[0] = fma(av[w], bv[w], part[0]);
        if (NS > 1) part[NS - 1] = fma(cv[w], dv[w], part[NS - 1]);
      }
      if ((cnt += W) >= kChunk) flush_parts<T, NS>(acc, part, cnt);
    }
  }
  for (long long i = tail + cm.first; i < n; i += cm.stride) {
    part[0] = fma(a[off + i], b[off + i], part[0]);
    if (NS > 1) part[NS - 1] = fma(c[off + i], d[off + i], part[NS - 1]);
    if (++cnt == kChunk) flush_parts<T, NS>(acc, part, cnt);
  }
  flush_parts<T, NS>(acc, part, cnt);
  block_reduce_finalize<NS>(red, acc);
}
template <typename T>
void launch_dot(const T* a, const T* b, const T* c, const T* d, long long n, const RedArgs& red,
                int nblocks, const int* halt, cudaStream_t st) {
  const int g = col_blocks(nblocks, red.ncol);
  const bool v = vec_ok<T>(n, red.ncol, {a, b, c, d});
  if (c) {
    if (v) dot_kernel<T, 2, true><<<g, 256, 0, st>>>(a, b, c, d, n, red, halt);
    else dot_kernel<T, 2, false><<<g, 256, 0, st>>>(a, b, c, d, n, red, halt);
  } else {
    if (v) dot_kernel<T, 1, true><<<g, 256, 0, st>>>(a, b, c, d, n, red, halt);
    else dot_kernel<T, 1, false><<<g, 256, 0, st>>>(a, b, c, d, n, red, halt);
  }
}

template <typename T, bool JAC, bool VEC>
__global__ void pcg_update_kernel(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                                  const T* __restrict__ p, const T* __restrict__ q,
                                  const T* __restrict__ dinv, long long n, RedArgs red,
                                  const PcgScalars* s) {
  const ColMap cm = colmap(red.ncol);
  if (*((volatile const int*)&s[cm.col].halt)) return;
  const T alpha = (T)s[cm.col].alpha;
  const long long off = (long long)cm.col * n;
  constexpr int NS = JAC ? 2 : 1;
  double acc[NS];
  T part[NS];
#pragma unroll
  for (int q2 = 0; q2 < NS; ++q2) acc[q2] = 0.0, part[q2] = T(0);
  int cnt = 0;
  long long tail = 0;
  if (VEC) {
    constexpr int W = V16<T>::W;
    const long long nv = n / W;
    tail = nv * W;
    for (long long i = cm.first; i < nv; i += cm.stride) {
      T xv[W], rv[W], pv[W], qv[W], dv[W], zv[W];
      ldv(x + off, i, xv);
      ldv(r + off, i, rv);
      ldv(p + off, i, pv);
      ldv(q + off, i, qv);
      if (JAC) ldv(dinv, i, dv);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        xv[w] = fma(alpha, pv[w], xv[w]);
        rv[w] = fma(-alpha, qv[w], rv[w]);
        part[0] = fma(rv[w], rv[w], part[0]);
        if (JAC) {
          zv[w] = rv[w] * dv[w];
          part[NS - 1] = fma(rv[w], zv[w], part[NS - 1]);
        }
      }
      stv(x + off, i, xv);
      stv(r + off, i, rv);
      if (JAC) stv(z + off, i, zv);
      if ((cnt += W) >= kChunk) flush_parts<T, NS>(acc, part, cnt);
    }
  }
  for (long long i = tail + cm.first; i < n; i += cm.stride) {
    const long long k = off + i;
    x[k] = fma(alpha, p[k], x[k]);
    const T ri = fma(-alpha, q[k], r[k]);
    r[k] = ri;
    part[0] = fma(ri, ri, part[0]);
    if (JAC) {
      const T zi = ri * dinv[i];  // the diagonal is shared by the columns
      z[k] = zi;
      part[NS - 1] = fma(ri, zi, part[NS - 1]);
    }
    if (++cnt == kChunk) flush_parts<T, NS>(acc, part, cnt);
  }
  flush_parts<T, NS>(acc, part, cnt);
  block_reduce_finalize<NS>(red, acc);
}
template <typename T>
void launch_pcg_update(T* x, T* r, T* z, const T* p, const T* q, const T* dinv, long long n,
                       const RedArgs& red, int nblocks, const PcgScalars* s, cudaStream_t st) {
  const int g = col_blocks(nblocks, red.ncol);
  const bool v = vec_ok<T>(n, red.ncol, {x, r, z, p, q, dinv}) && (red.ncol <= 1 || !dinv);
  if (dinv) {
    if (v) pcg_update_kernel<T, true, true><<<g, 256, 0, st>>>(x, r, z, p, q, dinv, n, red, s);
    else pcg_update_kernel<T, true, false><<<g, 256, 0, st>>>(x, r, z, p, q, dinv, n, red, s);
  } else {
    if (v) pcg_update_kernel<T, false, true><<<g, 256, 0, st>>>(x, r, z, p, q, dinv, n, red, s);
    else pcg_update_kernel<T, false, false><<<g, 256, 0, st>>>(x, r, z, p, q, dinv, n, red, s);
  }
}

// Flexible-PCG update: x += alpha p, r -= alpha q, sums ||r||^2 and r.z_old
// (the z of the previous iteration; its partner r.z_new comes from the
// V-cycle's last smoothing step).
template <typename T, bool VEC>
__global__ void pcg_update_mg_kernel(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                                     const T* __restrict__ q, const T* __restrict__ zo, long long n, RedArgs red,
                                     const PcgScalars* s) {
  const ColMap cm = colmap(red.ncol);
  if (*((volatile const int*)&s[cm.col].halt)) return;
  const T alpha = (T)s[cm.col].alpha;
  double acc[2] = {0.0, 0.0};
  T part[2] = {T(0), T(0)};
  int cnt = 0;
  long long tail = 0;
  if (VEC) {
    constexpr int W = V16<T>::W;
    const long long nv = n / W;
    tail = nv * W;
    for (long long i = cm.first; i < nv; i += cm.stride) {
      T xv[W], rv[W], pv[W], qv[W], zv[W];
      ldv(x, i, xv);
      ldv(r, i, rv);
      ldv(p, i, pv);
      ldv(q, i, qv);
      ldv(zo, i, zv);
#pragma unroll
      for (int w = 0; w < W; ++w) {
        xv[w] = fma(alpha, pv[w], xv[w]);
        rv[w] = fma(-alpha, qv[w], rv[w]);
        part[0] = fma(rv[w], rv[w], part[0]);
        part[1] = fma(rv[w], zv[w], part[1]);
      }
      stv(x, i, xv);
      stv(r, i, rv);
      if ((cnt += W) >= kChunk) flush_parts<T, 2>(acc, part, cnt);
    }
  }
  for (long long i = tail + cm.first; i < n; i += cm.stride) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    part[0] = fma(ri, ri, part[0]);
    part[1] = fma(ri, zo[i], part[1]);
    if (++cnt == kChunk) flush_parts<T, 2>(acc, part, cnt);
  }
  flush_parts<T, 2>(acc, part, cnt);
  block_reduce_finalize<2>(red, acc);
}
template <typename T>
void launch_pcg_update_mg(T* x, T* r, const T* p, const T* q, const T* zo, long long n, const RedArgs& red,
                          int nblocks, const PcgScalars* s, cudaStream_t st) {
  if (vec_ok<T>(n, 1, {x, r, p, q, zo}))
    pcg_update_mg_kernel<T, true><<<nblocks, 256, 0, st>>>(x, r, p, q, zo, n, red, s);
  else
    pcg_update_mg_kernel<T, false><<<nblocks, 256, 0, st>>>(x, r, p, q, zo, n, red, s);
}

template <typename T, bool VEC>
__global__ void p_update_kernel(T* __restrict__ p, const T* __restrict__ z, long long n,
                                const PcgScalars* s, int ncol) {
  const ColMap cm = colmap(ncol);
  if (*((volatile const int*)&s[cm.col].halt)) return;
  const T beta = (T)s[cm.col].beta;
  const long long off = (long long)cm.col * n;
  long long tail = 0;
  if (VEC) {
    constexpr int W = V16<T>::W;
    const long long nv = n / W;
    tail = nv * W;
    for (long long i = cm.first; i < nv; i += cm.stride) {
      T pv[W], zv[W];
      ldv(p + off, i, pv);
      ldv(z + off, i, zv);
#pragma unroll
      for (int w = 0; w < W; ++w) pv[w] = fma(beta, pv[w], zv[w]);
      stv(p + off, i, pv);
    }
  }
  for (long long i = tail + cm.first; i < n; i += cm.stride) p[off + i] = fma(beta, p[off + i], z[off + i]);
}
template <typename T>
void launch_p_update(T* p, const T* z, long long n, const PcgScalars* s, cudaStream_t st, int ncol) {
  if (vec_ok<T>(n, ncol, {p, z})) p_update_kernel<T, true><<<col_blocks(vec_blocks(n), ncol), 256, 0, st>>>(p, z, n, s, ncol);
  else p_update_kernel<T, false><<<col_blocks(vec_blocks(n), ncol), 256, 0, st>>>(p, z, n, s, ncol);
}

template <typename T>
__global__ void jacobi_precond_kernel(T* __restrict__ z, const T* __restrict__ r,
                                      const T* __restrict__ dinv, long long n, RedArgs red,
                                      const int* halt) {
  const ColMap cm = colmap(red.ncol);
  if (halted(halt, cm.col)) return;
  const long long off = (long long)cm.col * n;
  double acc[1] = {0.0};
  T part[1] = {T(0)};
  int cnt = 0;
  for (long long i = cm.first; i < n; i += cm.stride) {
    const T zi = r[off + i] * dinv[i];
    z[off + i] = zi;
    part[0] = fma(r[off + i], zi, part[0]);
    if (++cnt == kChunk) flush_parts<T, 1>(acc, part, cnt);
  }
  flush_parts<T, 1>(acc, part, cnt);
  block_reduce_finalize<1>(red, acc);
}
template <typename T>
void launch_jacobi_precond(T* z, const T* r, const T* dinv, long long n, const RedArgs& red,
                           int nblocks, const int* halt, cudaStream_t st) {
  jacobi_precond_kernel<T><<<col_blocks(nblocks, red.ncol), 256, 0, st>>>(z, r, dinv, n, red, halt);
}

// Column c of the batched vectors: dst = (T32)(src * scale[c]).
__global__ void scale_to_f32_kernel(float* __restrict__ d, const double* __restrict__ s,
                                    const double* scale, long long n, int ncol) {
  const ColMap cm = colmap(ncol);
  const double sc = scale[cm.col];
  const long long off = (long long)cm.col * n;
  for (long long i = cm.first; i < n; i += cm.stride) d[off + i] = (float)(s[off + i] * sc);
}
void launch_scale_to_f32(float* dst, const double* src, const double* scale, long long n,
                         cudaStream_t st, int ncol) {
  scale_to_f32_kernel<<<col_blocks(vec_blocks(n), ncol), 256, 0, st>>>(dst, src, scale, n, ncol);
}

// u += d / scale[c] per column
__global__ void add_scaled_f32_kernel(double* __restrict__ u, const float* __restrict__ d,
                                      const double* scale, long long n, int ncol) {
  const ColMap cm = colmap(ncol);
  const double inv = 1.0 / scale[cm.col];
  const long long off = (long long)cm.col * n;
  for (long long i = cm.first; i < n; i += cm.stride) u[off + i] = fma((double)d[off + i], inv, u[off + i]);
}
void launch_add_scaled_f32(double* u, const float* d, const double* scale, long long n,
                           cudaStream_t st, int ncol) {
  add_scaled_f32_kernel<<<col_blocks(vec_blocks(n), ncol), 256, 0, st>>>(u, d, scale, n, ncol);
}

template <typename T>
__global__ void axpby_kernel(T* __restrict__ x, T a, const T* __restrict__ y, T b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = a * x[i] + b * y[i];
}
template <typename T>
void launch_axpby(T* x, T a, const T* y, T b, long long n, cudaStream_t st) {
  axpby_kernel<T><<<vec_blocks(n), 256, 0, st>>>(x, a, y, b, n);
}

template <typename TD, typename TS>
__global__ void convert_kernel(TD* __restrict__ d, const TS* __restrict__ s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d[i] = (TD)s[i];
}
template <typename TD, typename TS>
void launch_convert(TD* dst, const TS* src, long long n, cudaStream_t st) {
  convert_kernel<TD, TS><<<vec_blocks(n), 256, 0, st>>>(dst, src, n);
}

// Reset the scalars of a nested (coarse-level) PCG: no convergence test,
// a fixed iteration count, and the parent's halt flag so a halted outer
// iteration skips the nested one too.
__global__ void scalars_init_kernel(PcgScalars* s0, const PcgScalars* parent, int max_iter, int ncol) {
  const int c = threadIdx.x;
  if (c >= ncol) return;
  PcgScalars* s = s0 + c;
  s->rz = 0.0; s->rz_prev = 0.0; s->pAp = 0.0; s->alpha = 0.0; s->beta = 0.0; s->rr = 0.0;
  s->bnorm = 1.0; s->relres = 0.0; s->best_rel = INFINITY; s->tol = 0.0;
  s->halt = parent ? *((volatile const int*)&parent[c].halt) : 0;
  s->status = 0; s->iter = 0; s->max_iter = max_iter; s->cadence = 0; s->test_now = 0;
}
void launch_scalars_init(PcgScalars* s, const PcgScalars* parent, int max_iter, cudaStream_t st, int ncol) {
  scalars_init_kernel<<<1, 64, 0, st>>>(s, parent, max_iter, ncol);
}

// ------------------------------------------------------------ batch passes
// Block b belongs to the instance whose [vblk0, vblk0 + vnblk) holds b; it
// strides over that instance's segment with the instance's block count.
__device__ __forceinline__ int batch_find_vec(const BatchInst* in, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (in[mid].vblk0 <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct BatchSeg {
  int id;
  long long off, n, first, stride, blk0, nblk;
};
__device__ __forceinline__ BatchSeg batch_seg(const BatchInst* in, int ninst, int node_sized) {
  const BatchInst& I = in[batch_find_vec(in, ninst, blockIdx.x)];
  BatchSeg sg;
  sg.id = I.id;
  sg.off = node_sized ? I.noff : I.off;
  sg.n = node_sized ? I.g.nnode() : I.g.ndof();
  sg.blk0 = I.vblk0;
  sg.nblk = I.vnblk;
  sg.first = (long long)(blockIdx.x - I.vblk0) * blockDim.x + threadIdx.x;
  sg.stride = (long long)I.vnblk * blockDim.x;
  return sg;
}
__device__ __forceinline__ bool inst_halted(const PcgScalars* s, int id) {
  return s && *((volatile const int*)&s[id].halt);
}

template <typename T, bool JAC>
__global__ void batch_pcg_update_kernel(const BatchInst* in, int ninst, int node_sized, T* __restrict__ x,
                                        T* __restrict__ r, T* __restrict__ z, const T* __restrict__ p,
                                        const T* __restrict__ q, const T* __restrict__ dinv, RedArgs red,
                                        const PcgScalars* s) {
  const BatchSeg sg = batch_seg(in, ninst, node_sized);
  if (inst_halted(s, sg.id)) return;
  const T alpha = (T)s[sg.id].alpha;
  constexpr int NS = JAC ? 2 : 1;
  double acc[NS];
  T part[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) acc[k] = 0.0, part[k] = T(0);
  int cnt = 0;
  for (long long i = sg.first; i < sg.n; i += sg.stride) {
    const long long k = sg.off + i;
    x[k] = fma(alpha, p[k], x[k]);
    const T ri = fma(-alpha, q[k], r[k]);
    r[k] = ri;
    part[0] = fma(ri, ri, part[0]);
    if (JAC) {
      const T zi = ri * dinv[k];
      z[k] = zi;
      part[NS - 1] = fma(ri, zi, part[NS - 1]);
    }
    if (++cnt == kChunk) flush_parts<T, NS>(acc, part, cnt);
  }
  flush_parts<T, NS>(acc, part, cnt);
  block_reduce_finalize_at<NS>(red, acc, sg.id, blockIdx.x, sg.nblk, sg.blk0, 1);
}
template <typename T>
void launch_batch_pcg_update(const BatchInst* in, int ninst, int nblocks, int node_sized, T* x, T* r, T* z,
                             const T* p, const T* q, const T* dinv, const RedArgs& red, const PcgScalars* s,
                             cudaStream_t st) {
  if (dinv) batch_pcg_update_kernel<T, true><<<nblocks, 256, 0, st>>>(in, ninst, node_sized, x, r, z, p, q, dinv, red, s);
  else batch_pcg_update_kernel<T, false><<<nblocks, 256, 0, st>>>(in, ninst, node_sized, x, r, z, p, q, dinv, red, s);
}

template <typename T>
__global__ void batch_p_update_kernel(const BatchInst* in, int ninst, int node_sized, T* __restrict__ p,
                                      const T* __restrict__ z, const PcgScalars* s) {
  const BatchSeg sg = batch_seg(in, ninst, node_sized);
  if (inst_halted(s, sg.id)) return;
  const T beta = (T)s[sg.id].beta;
  for (long long i = sg.first; i < sg.n; i += sg.stride) p[sg.off + i] = fma(beta, p[sg.off + i], z[sg.off + i]);
}
template <typename T>
void launch_batch_p_update(const BatchInst* in, int ninst, int nblocks, int node_sized, T* p, const T* z,
                           const PcgScalars* s, cudaStream_t st) {
  batch_p_update_kernel<T><<<nblocks, 256, 0, st>>>(in, ninst, node_sized, p, z, s);
}

template <typename T, int NS>
__global__ void batch_dot_kernel(const BatchInst* in, int ninst, int node_sized, const T* __restrict__ a,
                                 const T* __restrict__ b, const T* __restrict__ c, const T* __restrict__ d,
                                 RedArgs red, const PcgScalars* s) {
  const BatchSeg sg = batch_seg(in, ninst, node_sized);
  if (inst_halted(s, sg.id)) return;
  double acc[NS];
  T part[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) acc[k] = 0.0, part[k] = T(0);
  int cnt = 0;
  for (long long i = sg.first; i < sg.n; i += sg.stride) {
    const long long k = sg.off + i;
    part[0] = fma(a[k], b[k], part[0]);
    if (NS > 1) part[NS - 1] = fma(c[k], d[k], part[NS - 1]);
    if (++cnt == kChunk) flush_parts<T, NS>(acc, part, cnt);
  }
  flush_parts<T, NS>(acc, part, cnt);
  block_reduce_finalize_at<NS>(red, acc, sg.id, blockIdx.x, sg.nblk, sg.blk0, 1);
}
template <typename T>
void launch_batch_dot(const BatchInst* in, int ninst, int nblocks, int node_sized, const T* a, const T* b,
                      const T* c, const T* d, const RedArgs& red, const PcgScalars* s, cudaStream_t st) {
  if (c) batch_dot_kernel<T, 2><<<nblocks, 256, 0, st>>>(in, ninst, node_sized, a, b, c, d, red, s);
  else batch_dot_kernel<T, 1><<<nblocks, 256, 0, st>>>(in, ninst, node_sized, a, b, c, d, red, s);
}

template <typename T>
__global__ void batch_from64_kernel(const BatchInst* in, int ninst, T* __restrict__ dst,
                                    const double* __restrict__ src, const double* scale) {
  const BatchSeg sg = batch_seg(in, ninst, 0);
  const double sc = scale[sg.id];
  for (long long i = sg.first; i < sg.n; i += sg.stride) dst[sg.off + i] = (T)(src[sg.off + i] * sc);
}
template <typename T>
void launch_batch_from64(const BatchInst* in, int ninst, int nblocks, T* dst, const double* src,
                         const double* scale, cudaStream_t st) {
  batch_from64_kernel<T><<<nblocks, 256, 0, st>>>(in, ninst, dst, src, scale);
}

template <typename T>
__global__ void batch_accum_kernel(const BatchInst* in, int ninst, double* __restrict__ u, const T* __restrict__ d,
                                   const double* scale) {
  const BatchSeg sg = batch_seg(in, ninst, 0);
  const double sc = scale[sg.id];
  if (sc == 0.0) return;
  const double inv = 1.0 / sc;
  for (long long i = sg.first; i < sg.n; i += sg.stride) u[sg.off + i] = fma((double)d[sg.off + i], inv, u[sg.off + i]);
}
template <typename T>
void launch_batch_accum(const BatchInst* in, int ninst, int nblocks, double* u, const T* d, const double* scale,
                        cudaStream_t st) {
  batch_accum_kernel<T><<<nblocks, 256, 0, st>>>(in, ninst, u, d, scale);
}

__global__ void batch_set_beta_kernel(PcgScalars* s, const double* coef, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) s[i].beta = s[i].rz * coef[i];
}
void launch_batch_set_beta(PcgScalars* s, const double* coef, int n, cudaStream_t st) {
  batch_set_beta_kernel<<<(n + 127) / 128, 128, 0, st>>>(s, coef, n);
}

int vec_batch_plan(BatchInst* in, int n, int unit, int max_blocks) {
  auto units = [&](const BatchInst& b) -> long long {
    switch (unit) {
      case 1: return b.g.nnode();
      case 2: return b.g.nelem();
      case 3: return b.g2.nnode();
      default: return b.g.ndof();
    }
  };
  long long total = 0;
  for (int i = 0; i < n; ++i) total += units(in[i]);
  const double per = std::max(256.0, (double)total / std::max(1, max_blocks));
  int blk = 0;
  for (int i = 0; i < n; ++i) {
    const long long u = units(in[i]);
    const long long want = (long long)std::ceil((double)u / per);
    in[i].vblk0 = blk;
    in[i].vnblk = (int)std::max<long long>(1, std::min<long long>((u + 255) / 256, want));
    blk += in[i].vnblk;
  }
  return blk;
}

#define INST(T)                                                                                 \
  template void launch_fill<T>(T*, T, long long, cudaStream_t);                                 \
  template void launch_copy<T>(T*, const T*, long long, cudaStream_t);                          \
  template void launch_diag<T>(const Grid&, const Mask&, const T*, const ModalK<T>&, int, T, T*, \
                               T*, cudaStream_t);                                               \
  template void launch_dot<T>(const T*, const T*, const T*, const T*, long long, const RedArgs&, \
                              int, const int*, cudaStream_t);                                   \
  template void launch_pcg_update<T>(T*, T*, T*, const T*, const T*, const T*, long long,        \
                                     const RedArgs&, int, const PcgScalars*, cudaStream_t);      \
  template void launch_p_update<T>(T*, const T*, long long, const PcgScalars*, cudaStream_t, int); \
  template void launch_pcg_update_mg<T>(T*, T*, const T*, const T*, const T*, long long, const RedArgs&, int,  \
                                        const PcgScalars*, cudaStream_t);                                     \
  template void launch_jacobi_precond<T>(T*, const T*, const T*, long long, const RedArgs&, int, \
                                         const int*, cudaStream_t);                             \
  template void launch_axpby<T>(T*, T, const T*, T, long long, cudaStream_t);                    \
  template void launch_batch_pcg_update<T>(const BatchInst*, int, int, int, T*, T*, T*, const T*, const T*, \
                                           const T*, const RedArgs&, const PcgScalars*, cudaStream_t);      \
  template void launch_batch_p_update<T>(const BatchInst*, int, int, int, T*, const T*, const PcgScalars*,  \
                                         cudaStream_t);                                                     \
  template void launch_batch_dot<T>(const BatchInst*, int, int, int, const T*, const T*, const T*, const T*, \
                                    const RedArgs&, const PcgScalars*, cudaStream_t);                       \
  template void launch_batch_from64<T>(const BatchInst*, int, int, T*, const double*, const double*,        \
                                       cudaStream_t);                                                       \
  template void launch_batch_accum<T>(const BatchInst*, int, int, double*, const T*, const double*,         \
                                      cudaStream_t);
INST(double)
INST(float)
#undef INST
template void launch_mask_copy<double, double>(const Grid&, const Mask&, double*, const double*,
                                               cudaStream_t);
template void launch_mask_copy<float, float>(const Grid&, const Mask&, float*, const float*,
                                             cudaStream_t);
template void launch_mask_copy<double, float>(const Grid&, const Mask&, double*, const float*,
                                              cudaStream_t);
template void launch_mask_copy<float, double>(const Grid&, const Mask&, float*, const double*,
                                              cudaStream_t);
template void launch_convert<float, double>(float*, const double*, long long, cudaStream_t);
template void launch_convert<double, float>(double*, const float*, long long, cudaStream_t);

}  // namespace hexa
