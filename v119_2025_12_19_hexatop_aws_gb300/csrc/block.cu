// Block PCG kernels: k right-hand sides held as k consecutive columns of
// length n (column j of X starts at X + j*n).
//
// One block iteration (O'Leary's block CG in its flexible form) is
//   Z = M R                      (preconditioner, column by column)
//   D = Q^T Z,  beta = -G^+ D    (gram + k x k solve; G = P^T A P of the last step)
//   P = Z + P beta               (block_p_update)
//   Q = A P                      (the multi-column operator)
//   G = P^T Q, C = P^T R         (gram with two right operands)
//   alpha = G^+ C                (k x k solve)
//   X += P alpha, R -= Q alpha   (block_update, with the column norms of R)
// G^+ is a pseudo-inverse through a Cholesky factorisation that drops a
// direction whose pivot is below eps * G_jj (a search direction dependent on
// the others), so converged or dependent columns cannot break the iteration.
#include <cuda_runtime.h>

#include <algorithm>

#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

namespace {

constexpr int kThreads = 256;
constexpr int kGramFold = 8;  // tiles summed in T before one fold into the FP64 accumulators

template <typename T>
constexpr int gram_td() { return sizeof(T) == 8 ? 64 : 128; }

template <int KC, int NB>
struct GramShape {
  static constexpr int NBC = NB * KC;            // right operand columns
  static constexpr int RI = KC >= 2 ? 2 : 1;     // register block of a thread
  static constexpr int RJ = NBC >= 4 ? 4 : NBC;
  static constexpr int GI = KC / RI, GJ = NBC / RJ, GROUPS = GI * GJ;
  static constexpr int SLICES = kThreads / GROUPS;  // DOF slices of a tile
  static constexpr int NPAIR = KC * NBC;
};

__device__ __forceinline__ bool halt_set(const int* h) { return h && *((volatile const int*)h); }

// out[i * NBC + j] = sum_d a_i[d] * b_j[d] for i < KC, j < NBC, where
// b_j = b1_j for j < KC and b2_{j-KC} otherwise; columns >= k read as zero.
// Tiles of TD DOFs are staged in shared memory (a warp loads one column's TD
// consecutive values: coalesced, shift-and-mask indexing); each thread
// accumulates an RI x RJ block of pairs over one DOF slice in T across
// kGramFold tiles before folding into FP64 -- GB300's FP64 rate is a small
// fraction of its FP32 rate, and folding every tile made the pass FP64-bound.
// Per-block partials are summed in block order by the last block (ticket):
// the result is bitwise reproducible.
template <typename T, int KC, int NB>
__global__ void __launch_bounds__(kThreads) gram_kernel(const T* __restrict__ a, const T* __restrict__ b1,
                                                         const T* __restrict__ b2, int k, long long n,
                                                         double* partials, unsigned* ticket, double* out,
                                                         const int* halt) {
  if (halt_set(halt)) return;
  using S = GramShape<KC, NB>;
  constexpr int TD = gram_td<T>();
  __shared__ T sA[KC][TD + 1];
  __shared__ T sB[S::NBC][TD + 1];
  __shared__ double sred[S::SLICES][S::NPAIR];
  __shared__ bool am_last;
  const int tid = threadIdx.x;
  const int grp = tid % S::GROUPS, slice = tid / S::GROUPS;
  const int gi = grp / S::GJ, gj = grp % S::GJ;
  double acc[S::RI][S::RJ];
#pragma unroll
  for (int i = 0; i < S::RI; ++i)
#pragma unroll
    for (int j = 0; j < S::RJ; ++j) acc[i][j] = 0.0;
  static_assert((TD & (TD - 1)) == 0, "TD is a power of two");
  constexpr int TDLOG = TD == 128 ? 7 : 6;
  const long long ntiles = (n + TD - 1) / TD;
  T part[S::RI][S::RJ];
#pragma unroll
  for (int i = 0; i < S::RI; ++i)
#pragma unroll
    for (int j = 0; j < S::RJ; ++j) part[i][j] = T(0);
  int folded = 0;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long long d0 = t * TD;
    const bool full = d0 + TD <= n;
#pragma unroll 4
    for (int e = tid; e < (KC + S::NBC) * TD; e += kThreads) {
      const int col = e >> TDLOG, d = e & (TD - 1);
      const long long gd = d0 + d;
      const bool in = full || gd < n;
      if (col < KC) {
        sA[col][d] = (col < k && in) ? a[(long long)col * n + gd] : T(0);
      } else {
        const int cb = col - KC, j = cb < KC ? cb : cb - KC;
        const T* src = cb < KC ? b1 : b2;
        sB[cb][d] = (j < k && in) ? src[(long long)j * n + gd] : T(0);
      }
    }
    __syncthreads();
    for (int d = slice; d < TD; d += S::SLICES) {
      T av[S::RI], bv[S::RJ];
#pragma unroll
      for (int i = 0; i < S::RI; ++i) av[i] = sA[gi * S::RI + i][d];
#pragma unroll
      for (int j = 0; j < S::RJ; ++j) bv[j] = sB[gj * S::RJ + j][d];
#pragma unroll
      for (int i = 0; i < S::RI; ++i)
#pragma unroll
        for (int j = 0; j < S::RJ; ++j) part[i][j] = fma(av[i], bv[j], part[i][j]);
    }
    if (++folded == kGramFold) {
      folded = 0;
#pragma unroll
      for (int i = 0; i < S::RI; ++i)
#pragma unroll
        for (int j = 0; j < S::RJ; ++j) acc[i][j] += (double)part[i][j], part[i][j] = T(0);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < S::RI; ++i)
#pragma unroll
    for (int j = 0; j < S::RJ; ++j)
      sred[slice][(gi * S::RI + i) * S::NBC + gj * S::RJ + j] = acc[i][j] + (double)part[i][j];
  __syncthreads();
  for (int p = tid; p < S::NPAIR; p += kThreads) {
    double s = 0.0;
    for (int sl = 0; sl < S::SLICES; ++sl) s += sred[sl][p];
    partials[(long long)blockIdx.x * S::NPAIR + p] = s;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (int p = tid; p < S::NPAIR; p += kThreads) {
    double s = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) s += ((volatile double*)partials)[(long long)b * S::NPAIR + p];
    out[p] = s;
  }
  if (tid == 0) *ticket = 0u;
}

// The same sums for FP32 columns as a streaming pass: each thread walks its
// grid-stride DOFs with coalesced loads (consecutive lanes, consecutive DOFs
// of one column) and keeps its KC x NJ column-pair sums in registers, NJ =
// NBC / H columns of the right operand per thread (H = 2 threads per DOF when
// NBC = 16, so that the sums fit in registers).  No shared-memory staging and
// no per-tile FP64 work: GB300's FP64 rate is a small fraction of its FP32
// rate.  Each thread's FP32 sums (a few hundred products at the sizes this
// path serves) are folded into FP64 once, at the end, reduced over the warp by
// shuffles and over the block in shared memory, and the per-block partials
// are summed in block order by the last block (ticket): bitwise reproducible.
template <int KC, int NB>
__global__ void __launch_bounds__(kThreads, 2) gram_stream_kernel(const float* __restrict__ a, const float* __restrict__ b1,
                                                                   const float* __restrict__ b2, int k, long long n,
                                                                   double* partials, unsigned* ticket, double* out,
                                                                   const int* halt) {
  if (halt_set(halt)) return;
  constexpr int NBC = NB * KC, H = NBC > 8 ? 2 : 1, NJ = NBC / H, NPAIR = KC * NBC, NW = kThreads / 32;
  __shared__ double sw[NW][NPAIR];
  __shared__ bool am_last;
  const int tid = threadIdx.x, h = tid % H, lane = tid & 31, warp = tid >> 5;
  float acc[KC][NJ];
#pragma unroll
  for (int i = 0; i < KC; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j) acc[i][j] = 0.f;
  const long long stride = (long long)gridDim.x * (kThreads / H);
#pragma unroll 2
  for (long long d = ((long long)blockIdx.x * kThreads + tid) / H; d < n; d += stride) {
    float av[KC], bv[NJ];
#pragma unroll
    for (int i = 0; i < KC; ++i) av[i] = i < k ? __ldg(a + (long long)i * n + d) : 0.f;
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      const int col = h * NJ + j, jj = col < KC ? col : col - KC;
      const float* src = col < KC ? b1 : b2;
      bv[j] = jj < k ? __ldg(src + (long long)jj * n + d) : 0.f;
    }
#pragma unroll
    for (int i = 0; i < KC; ++i)
#pragma unroll
      for (int j = 0; j < NJ; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
  }
  // warp: lanes of the same h (offsets that are multiples of H)
#pragma unroll
  for (int i = 0; i < KC; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      double v = (double)acc[i][j];
#pragma unroll
      for (int off = 16; off >= H; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (lane < H) sw[warp][i * NBC + lane * NJ + j] = v;
    }
  __syncthreads();
  for (int q = tid; q < NPAIR; q += kThreads) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) v += sw[w][q];
    partials[(long long)blockIdx.x * NPAIR + q] = v;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (int q = tid; q < NPAIR; q += kThreads) {
    double v = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) v += ((volatile double*)partials)[(long long)b * NPAIR + q];
    out[q] = v;
  }
  if (tid == 0) *ticket = 0u;
}

// out (k x k, row = direction, column = right-hand side) = sign * G^+ rhs with
// G_ij = (g[i*ldg+j] + g[j*ldg+i]) / 2 and rhs_ij = r[i*ldr + roff + j].
__global__ void block_solve_kernel(const double* g, int ldg, const double* r, int ldr, int roff, int k, double sign,
                                   double eps, double* out, const int* halt) {
  if (halt_set(halt)) return;
  __shared__ double L[kMaxBlockCols][kMaxBlockCols];
  __shared__ int drop[kMaxBlockCols];
  const int t = threadIdx.x;
  if (t == 0) {
    for (int j = 0; j < k; ++j) {
      const double gjj = g[j * ldg + j];
      double d = gjj;
      for (int m = 0; m < j; ++m) d -= L[j][m] * L[j][m];
      const bool ok = (gjj > 0.0) && (d > eps * gjj) && (d == d);
      drop[j] = ok ? 0 : 1;
      const double ljj = ok ? sqrt(d) : 0.0;
      L[j][j] = ljj;
      for (int i = j + 1; i < k; ++i) {
        double v = 0.5 * (g[i * ldg + j] + g[j * ldg + i]);
        for (int m = 0; m < j; ++m) v -= L[i][m] * L[j][m];
        L[i][j] = ok ? v / ljj : 0.0;
      }
      for (int i = 0; i < j; ++i) L[i][j] = 0.0;
    }
  }
  __syncthreads();
  if (t < k) {
    double y[kMaxBlockCols];
    for (int i = 0; i < k; ++i) {  // L y = rhs(:, t)
      double v = r[i * ldr + roff + t];
      for (int m = 0; m < i; ++m) v -= L[i][m] * y[m];
      y[i] = drop[i] ? 0.0 : v / L[i][i];
    }
    for (int i = k - 1; i >= 0; --i) {  // L^T x = y
      double v = y[i];
      for (int m = i + 1; m < k; ++m) v -= L[m][i] * y[m];
      y[i] = drop[i] ? 0.0 : v / L[i][i];
    }
    for (int i = 0; i < k; ++i) out[i * k + t] = sign * y[i];
  }
}

// Row i of a k x k coefficient block in shared memory, read with vector
// loads inside the DOF loop.  The loads are volatile asm so the compiler does
// not hoist all k^2 coefficients into registers ahead of the loop.
template <typename T, int KC>
__device__ __forceinline__ void coef_row(const T* row, T (&a)[KC]) {
  const unsigned addr = (unsigned)__cvta_generic_to_shared(row);
  if constexpr (sizeof(T) == 4 && KC % 4 == 0) {
#pragma unroll
    for (int q = 0; q < KC / 4; ++q) {
      float x, y, z, w;
      asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                   : "=f"(x), "=f"(y), "=f"(z), "=f"(w)
                   : "r"(addr + 16u * q));
      a[4 * q] = x, a[4 * q + 1] = y, a[4 * q + 2] = z, a[4 * q + 3] = w;
    }
  } else if constexpr (sizeof(T) == 8 && KC % 2 == 0) {
#pragma unroll
    for (int q = 0; q < KC / 2; ++q) {
      double x, y;
      asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "r"(addr + 16u * q));
      a[2 * q] = x, a[2 * q + 1] = y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < KC; ++j) a[j] = row[j];
  }
}

// X_j += sum_i P_i alpha_ij ; R_j -= sum_i Q_i alpha_ij ; sums ||R_j||^2.
// A thread issues all 4k loads of its DOF before any arithmetic and reads
// the k x k coefficients as shared-memory rows (vector loads, the same
// address across the warp): at 8 columns the pass needs about 60 registers
// instead of holding 64 coefficients in registers at quarter occupancy.  The
// sums over i run in the same order as a per-column loop would.
template <typename T, int KC>
__global__ void __launch_bounds__(kThreads, KC <= 8 ? 3 : 1) block_update_kernel(T* __restrict__ X, T* __restrict__ R,
                                                                 const T* __restrict__ P, const T* __restrict__ Q,
                                                                 const double* alpha, int k, long long n,
                                                                 RedArgs red) {
  if (halt_set(red.s ? &red.s->halt : nullptr)) return;
  __shared__ __align__(16) T sa[KC][KC];
  for (int e = threadIdx.x; e < KC * KC; e += blockDim.x) {
    const int i = e / KC, j = e % KC;
    sa[i][j] = (i < k && j < k) ? (T)alpha[i * k + j] : T(0);
  }
  __syncthreads();
  double acc[KC];
  T part[KC];
#pragma unroll
  for (int j = 0; j < KC; ++j) acc[j] = 0.0, part[j] = T(0);
  int cnt = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long d = (long long)blockIdx.x * blockDim.x + threadIdx.x; d < n; d += stride) {
    T pv[KC], qv[KC], xv[KC], rv[KC];
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      const bool in = i < k;
      const long long o = (long long)i * n + d;
      pv[i] = in ? P[o] : T(0);
      qv[i] = in ? Q[o] : T(0);
      xv[i] = in ? X[o] : T(0);
      rv[i] = in ? R[o] : T(0);
    }
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      T ar[KC];
      coef_row<T, KC>(&sa[i][0], ar);
#pragma unroll
      for (int j = 0; j < KC; ++j) {
        xv[j] = fma(pv[i], ar[j], xv[j]);
        rv[j] = fma(-qv[i], ar[j], rv[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < KC; ++j) {
      if (j < k) {
        const long long o = (long long)j * n + d;
        X[o] = xv[j];
        R[o] = rv[j];
        part[j] = fma(rv[j], rv[j], part[j]);
      }
    }
    if (++cnt == 32) {
#pragma unroll
      for (int j = 0; j < KC; ++j) acc[j] += (double)part[j], part[j] = T(0);
      cnt = 0;
    }
  }
#pragma unroll
  for (int j = 0; j < KC; ++j) acc[j] += (double)part[j];
  block_reduce_finalize<KC>(red, acc);
}

// P_j = Z_j + sum_i P_i beta_ij (all 2k loads first, coefficients as
// shared-memory rows, like block_update_kernel)
template <typename T, int KC>
__global__ void __launch_bounds__(kThreads, KC <= 8 ? 4 : 1) block_p_update_kernel(T* __restrict__ P, const T* __restrict__ Z,
                                                                   const double* beta, int k, long long n,
                                                                   const int* halt) {
  if (halt_set(halt)) return;
  __shared__ __align__(16) T sb[KC][KC];
  for (int e = threadIdx.x; e < KC * KC; e += blockDim.x) {
    const int i = e / KC, j = e % KC;
    sb[i][j] = (i < k && j < k) ? (T)beta[i * k + j] : T(0);
  }
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long d = (long long)blockIdx.x * blockDim.x + threadIdx.x; d < n; d += stride) {
    T pv[KC], v[KC];
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      const bool in = i < k;
      pv[i] = in ? P[(long long)i * n + d] : T(0);
      v[i] = in ? Z[(long long)i * n + d] : T(0);
    }
#pragma unroll
    for (int i = 0; i < KC; ++i) {
      T br[KC];
      coef_row<T, KC>(&sb[i][0], br);
#pragma unroll
      for (int j = 0; j < KC; ++j) v[j] = fma(pv[i], br[j], v[j]);
    }
#pragma unroll
    for (int j = 0; j < KC; ++j)
      if (j < k) P[(long long)j * n + d] = v[j];
  }
}

// Column kernels: blockIdx.y is the column.
template <typename T>
__global__ void cols_jacobi_kernel(T* __restrict__ z, const T* __restrict__ r, const T* __restrict__ dinv,
                                   long long n, const int* halt) {
  if (halt_set(halt)) return;
  const long long off = (long long)blockIdx.y * n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[off + i] = r[off + i] * dinv[i];
}

template <typename T>
__global__ void cols_from64_kernel(T* __restrict__ d, const double* __restrict__ s, const double* scale, long long n) {
  const long long off = (long long)blockIdx.y * n;
  const double sc = scale[blockIdx.y];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[off + i] = (T)(s[off + i] * sc);
}

template <typename T>
__global__ void cols_accum_kernel(double* __restrict__ u, const T* __restrict__ d, const double* scale, long long n) {
  const long long off = (long long)blockIdx.y * n;
  const double sc = scale[blockIdx.y];
  if (sc == 0.0) return;  // frozen column: no correction
  const double inv = 1.0 / sc;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    u[off + i] = fma((double)d[off + i], inv, u[off + i]);
}

int col_grid_x(long long n, int k) {
  const long long want = std::max<long long>(1, 152LL * 8 / std::max(1, k));
  return (int)std::max<long long>(1, std::min<long long>((n + kThreads - 1) / kThreads, want));
}

}  // namespace

long long block_partials_needed(int k) {
  const int kc = k <= 1 ? 1 : k <= 2 ? 2 : k <= 4 ? 4 : k <= 8 ? 8 : 16;
  return (long long)kBlockRedBlocks * kc * 2 * kc + (long long)kBlockRedBlocks * kc;
}

int block_kc(int k) { return k <= 1 ? 1 : k <= 2 ? 2 : k <= 4 ? 4 : k <= 8 ? 8 : 16; }

template <typename T>
void launch_gram(const T* a, const T* b1, const T* b2, int k, long long n, double* partials, unsigned* ticket,
                 double* out, const int* halt, cudaStream_t st) {
  constexpr int TD = gram_td<T>();
  const int g = (int)std::max<long long>(1, std::min<long long>((n + TD - 1) / TD, kBlockRedBlocks));
  const int kc = block_kc(k);
#define HEXA_GRAM(KCV)                                                                                        \
  case KCV:                                                                                                  \
    if constexpr (sizeof(T) == 4 && (KCV == 4 || KCV == 8)) {                                                              \
      if (b2) gram_stream_kernel<KCV, 2><<<kBlockRedBlocks, kThreads, 0, st>>>(a, b1, b2, k, n, partials, ticket, out, halt); \
      else gram_stream_kernel<KCV, 1><<<kBlockRedBlocks, kThreads, 0, st>>>(a, b1, b2, k, n, partials, ticket, out, halt);   \
    } else if (b2) {                                                                                         \
      gram_kernel<T, KCV, 2><<<g, kThreads, 0, st>>>(a, b1, b2, k, n, partials, ticket, out, halt);          \
    } else {                                                                                                 \
      gram_kernel<T, KCV, 1><<<g, kThreads, 0, st>>>(a, b1, b2, k, n, partials, ticket, out, halt);          \
    }                                                                                                        \
    break;
  switch (kc) {
    HEXA_GRAM(1)
    HEXA_GRAM(2)
    HEXA_GRAM(4)
    HEXA_GRAM(8)
    HEXA_GRAM(16)
    default: break;
  }
#undef HEXA_GRAM
}

void launch_block_solve(const double* g, int ldg, const double* r, int ldr, int roff, int k, double sign, double eps,
                        double* out, const int* halt, cudaStream_t st) {
  block_solve_kernel<<<1, 32, 0, st>>>(g, ldg, r, ldr, roff, k, sign, eps, out, halt);
}

template <typename T>
void launch_block_update(T* X, T* R, const T* P, const T* Q, const double* alpha, int k, long long n,
                         const RedArgs& red, cudaStream_t st) {
  // one wave: three CTAs per SM fit (launch bounds) and the loop strides over n
  const int g = (int)std::max<long long>(1, std::min<long long>((n + kThreads - 1) / kThreads, 152LL * 3));
#define HEXA_BU(KCV) \
  case KCV: block_update_kernel<T, KCV><<<g, kThreads, 0, st>>>(X, R, P, Q, alpha, k, n, red); break;
  switch (block_kc(k)) {
    HEXA_BU(1)
    HEXA_BU(2)
    HEXA_BU(4)
    HEXA_BU(8)
    HEXA_BU(16)
    default: break;
  }
#undef HEXA_BU
}

template <typename T>
void launch_block_p_update(T* P, const T* Z, const double* beta, int k, long long n, const int* halt,
                           cudaStream_t st) {
  const int g = (int)std::max<long long>(1, std::min<long long>((n + kThreads - 1) / kThreads, 152LL * 4));
#define HEXA_BP(KCV) \
  case KCV: block_p_update_kernel<T, KCV><<<g, kThreads, 0, st>>>(P, Z, beta, k, n, halt); break;
  switch (block_kc(k)) {
    HEXA_BP(1)
    HEXA_BP(2)
    HEXA_BP(4)
    HEXA_BP(8)
    HEXA_BP(16)
    default: break;
  }
#undef HEXA_BP
}

template <typename T>
void launch_cols_jacobi(T* z, const T* r, const T* dinv, long long n, int k, const int* halt, cudaStream_t st) {
  cols_jacobi_kernel<T><<<dim3(col_grid_x(n, k), k), kThreads, 0, st>>>(z, r, dinv, n, halt);
}

template <typename T>
void launch_cols_from64(T* dst, const double* src, const double* scale, long long n, int k, cudaStream_t st) {
  cols_from64_kernel<T><<<dim3(col_grid_x(n, k), k), kThreads, 0, st>>>(dst, src, scale, n);
}

template <typename T>
void launch_cols_accum(double* u, const T* d, const double* scale, long long n, int k, cudaStream_t st) {
  cols_accum_kernel<T><<<dim3(col_grid_x(n, k), k), kThreads, 0, st>>>(u, d, scale, n);
}

#define HEXA_BLOCK_INST(T)                                                                                    \
  template void launch_gram<T>(const T*, const T*, const T*, int, long long, double*, unsigned*, double*,    \
                               const int*, cudaStream_t);                                                    \
  template void launch_block_update<T>(T*, T*, const T*, const T*, const double*, int, long long,            \
                                       const RedArgs&, cudaStream_t);                                         \
  template void launch_block_p_update<T>(T*, const T*, const double*, int, long long, const int*, cudaStream_t); \
  template void launch_cols_jacobi<T>(T*, const T*, const T*, long long, int, const int*, cudaStream_t);     \
  template void launch_cols_from64<T>(T*, const double*, const double*, long long, int, cudaStream_t);       \
  template void launch_cols_accum<T>(double*, const T*, const double*, long long, int, cudaStream_t);
HEXA_BLOCK_INST(float)
HEXA_BLOCK_INST(double)
#undef HEXA_BLOCK_INST

}  // namespace hexa
