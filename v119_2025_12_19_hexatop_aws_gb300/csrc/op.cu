// (a) Matrix-free hex8 elasticity operator, node-centric and deterministic.
//
// Replaces the reference's one-thread-per-element atomic scatter
// (src/Solvers/GPUSolver.jl:91-128, wrapped by apply_A! :322-330 with its
// expand/contract passes :146-160).  Here each CTA owns a 31 x (TYW-1) tile of
// node columns and marches through z.  Thread (lane, wy) owns the element
// column (i0-1+lane, j0-1+wy): at each element layer it forms the element's
// 24 modal coefficients from its 4 corner nodes of the two node layers
// (xy-Hadamard of the new layer, reused as the lower layer of the next step),
// applies the eight 3x3 modal blocks of K0 scaled by the element factor, and
// keeps the upper-layer half in registers as a carry for the next step.  The
// four columns around a node are summed with one warp shuffle (x) and one
// shared-memory exchange (y); no atomics anywhere, so y is bitwise
// reproducible.  Fixed DOFs are masked in-kernel (no free-DOF map), and the
// epilogue fuses the PCG dot, the residual b - Ax, a damped-Jacobi step or a
// Chebyshev step.
#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

// Structural zeros of the modal blocks (hold for every brick and every nu):
// single-bit classes q = 1<<c0 carry a rigid translation (row/column c0 zero);
// two-bit classes decouple the component whose bit is not in q.
__host__ __device__ constexpr bool modal_nz(int q, int c, int c2) {
  return ((q == 1) || (q == 2) || (q == 4))
             ? (c != (q == 1 ? 0 : (q == 2 ? 1 : 2)) && c2 != (q == 1 ? 0 : (q == 2 ? 1 : 2)))
         : ((q == 3) || (q == 5) || (q == 6))
             ? ((c == (q == 3 ? 2 : (q == 5 ? 1 : 0))) == (c2 == (q == 3 ? 2 : (q == 5 ? 1 : 0))))
             : true;
}

template <typename T>
__device__ __forceinline__ T ldx(const T* p) { return __ldg(p); }

// Corner cc = dx + 2*dy of the column (ie, je) at node layer kk; zeros outside.
template <typename T>
__device__ __forceinline__ void load_corners(const Grid& g, const T* __restrict__ x, int ie, int je,
                                             int kk, T (&v)[4][3]) {
  const bool kok = (kk >= 0) && (kk < g.NZ);
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const int i = ie + (cc & 1), j = je + (cc >> 1);
    const bool ok = kok && (i >= 0) && (i < g.NX) && (j >= 0) && (j < g.NY);
    const long long n = ok ? ((long long)i + (long long)g.NX * ((long long)j + (long long)g.NY * kk)) : 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) v[cc][c] = ok ? ldx(x + 3 * n + c) : T(0);
  }
}

// xy part of the Hadamard transform: corners (dx,dy) -> modes (mx,my), both
// indexed dx + 2*dy.
template <typename T>
__device__ __forceinline__ void xy_forward(const T (&v)[4][3], T (&m)[4][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const T a0 = v[0][c] + v[1][c], a1 = v[1][c] - v[0][c];
    const T b0 = v[2][c] + v[3][c], b1 = v[3][c] - v[2][c];
    m[0][c] = a0 + b0;
    m[1][c] = a1 + b1;
    m[2][c] = b0 - a0;
    m[3][c] = b1 - a1;
  }
}

// Transpose of xy_forward: modes -> corner values.
template <typename T>
__device__ __forceinline__ void xy_inverse(const T (&m)[4][3], T (&v)[4][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const T A0 = m[0][c] - m[2][c], B0 = m[0][c] + m[2][c];
    const T A1 = m[1][c] - m[3][c], B1 = m[1][c] + m[3][c];
    v[0][c] = A0 - A1;
    v[1][c] = A0 + A1;
    v[2][c] = B0 - B1;
    v[3][c] = B0 + B1;
  }
}

// One element: lower/upper xy-modal node data -> lower/upper xy-modal
// contributions of f * K0 * u_e.
template <typename T>
__device__ __forceinline__ void element_modal(const ModalK<T>& K, const T (&L)[4][3],
                                              const T (&U)[4][3], T f, T (&lo)[4][3], T (&hi)[4][3]) {
  T uh[8][3];
#pragma unroll
  for (int mxy = 0; mxy < 4; ++mxy)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      uh[mxy][c] = L[mxy][c] + U[mxy][c];
      uh[mxy + 4][c] = U[mxy][c] - L[mxy][c];
    }
  T wh[8][3];
#pragma unroll
  for (int m = 0; m < 8; ++m)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int q = m ^ (1 << c);
      T s = T(0);
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        if (modal_nz(q, c, c2)) s = fma(K.B[q][c][c2], uh[q ^ (1 << c2)][c2], s);
      wh[m][c] = s * f;
    }
#pragma unroll
  for (int mxy = 0; mxy < 4; ++mxy)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[mxy][c] = wh[mxy][c] - wh[mxy + 4][c];
      hi[mxy][c] = wh[mxy][c] + wh[mxy + 4][c];
    }
}

template <typename T, int MODE, int TYW>
__global__ void __launch_bounds__(32 * TYW) op_kernel(const OpArgs<T> a) {
  if (a.halt && *((volatile const int*)a.halt)) return;
  constexpr int NX_OWN = 31, NY_OWN = TYW - 1;
  constexpr bool NEED_F = (MODE == OP_JACOBI || MODE == OP_CHEB2);
  __shared__ T xch[2][TYW][32][NEED_F ? 4 : 3];

  const Grid g = a.g;
  const int lane = threadIdx.x, wy = threadIdx.y;
  const int i0 = blockIdx.x * NX_OWN, j0 = blockIdx.y * NY_OWN;
  const int k0 = blockIdx.z * a.kchunk;
  const int k1 = min(k0 + a.kchunk, g.NZ);
  const int ie = i0 - 1 + lane, je = j0 - 1 + wy;
  const bool colv = (ie >= 0) && (ie < g.nx) && (je >= 0) && (je < g.ny);
  const long long ecol = colv ? ((long long)ie + (long long)g.nx * je) : 0;
  const long long eplane = (long long)g.nx * g.ny;
  const int in = i0 + lane, jn = j0 + wy;
  const bool own = (lane < NX_OWN) && (wy < NY_OWN) && (in < g.NX) && (jn < g.NY);
  const T* __restrict__ x = a.x;
  const T* __restrict__ fac = a.fac;

  auto facload = [&](int k) -> T {
    return (colv && k >= 0 && k < g.nz) ? ldx(fac + ecol + eplane * k) : T(0);
  };

  T Lm[4][3], carry[4][3], xown[3];
  T fprev;
  {
    T raw[4][3];
    load_corners<T>(g, x, ie, je, k0 - 1, raw);
    T Lprev[4][3];
    xy_forward<T>(raw, Lprev);
    load_corners<T>(g, x, ie, je, k0, raw);
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
    xy_forward<T>(raw, Lm);
    fprev = facload(k0 - 1);
    T lo[4][3];
    element_modal<T>(a.K, Lprev, Lm, fprev, lo, carry);
  }

  double acc0 = 0.0;
  T nraw[4][3];
  load_corners<T>(g, x, ie, je, k0 + 1, nraw);
  T fnext = facload(k0);

  for (int k = k0; k < k1; ++k) {
    T raw[4][3];
#pragma unroll
    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
      for (int c = 0; c < 3; ++c) raw[cc][c] = nraw[cc][c];
    const T f = fnext;
    if (k + 1 < k1) {  // prefetch the next layer
      load_corners<T>(g, x, ie, je, k + 2, nraw);
      fnext = facload(k + 1);
    }
    T Um[4][3];
    xy_forward<T>(raw, Um);
    T lo[4][3], hi[4][3];
    element_modal<T>(a.K, Lm, Um, f, lo, hi);
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        lo[m][c] += carry[m][c];
        carry[m][c] = hi[m][c];
        Lm[m][c] = Um[m][c];
      }
    T cv[4][3];
    xy_inverse<T>(lo, cv);
    // node (i0+p, j0+q) = c11(p,q) + c01(p+1,q) + c10(p,q+1) + c00(p+1,q+1)
    T T1[3], T0[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T1[c] = cv[3][c] + __shfl_down_sync(0xffffffffu, cv[2][c], 1);
      T0[c] = cv[1][c] + __shfl_down_sync(0xffffffffu, cv[0][c], 1);
    }
    T F1 = T(0);
    if (NEED_F) {
      const T fcol = fprev + f;
      F1 = fcol + __shfl_down_sync(0xffffffffu, fcol, 1);
    }
    fprev = f;
    const int buf = k & 1;
#pragma unroll
    for (int c = 0; c < 3; ++c) xch[buf][wy][lane][c] = T0[c];
    if (NEED_F) xch[buf][wy][lane][NEED_F ? 3 : 0] = F1;
    __syncthreads();
    if (own) {
      const long long n = (long long)in + (long long)g.NX * ((long long)jn + (long long)g.NY * k);
      const unsigned fx = fixed_bits(g, a.m, in, jn, k, n);
      T Kx[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) Kx[c] = T1[c] + xch[buf][wy + 1][lane][c];
      T fsum = T(0);
      if (NEED_F) fsum = F1 + xch[buf][wy + 1][lane][NEED_F ? 3 : 0];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const bool fixd = (fx >> c) & 1u;
        const T Ax = fma(a.sigma, xown[c], Kx[c]);
        T out;
        if (MODE == OP_APPLY) {
          out = fixd ? T(0) : Ax;
        } else if (MODE == OP_APPLY_DOT) {
          out = fixd ? T(0) : Ax;
          acc0 += (double)xown[c] * (double)out;
        } else if (MODE == OP_RESID || MODE == OP_RESID_NORM) {
          out = fixd ? T(0) : (ldx(a.b + 3 * n + c) - Ax);
          if (MODE == OP_RESID_NORM) acc0 += (double)out * (double)out;
        } else if (MODE == OP_JACOBI) {  // x + omega (b - Ax) / D
          const T d = fma(a.K.dd[a.diag_quirk ? 0 : c], fsum, a.sigma);
          out = fixd ? T(0) : fma(a.omega, (ldx(a.b + 3 * n + c) - Ax) / d, xown[c]);
        } else {  // OP_CHEB2: x + c1 (x - x_prev) + c2 D^-1 (b - Ax)
          const T d = fma(a.K.dd[a.diag_quirk ? 0 : c], fsum, a.sigma);
          const T xp = a.xin ? a.xin[3 * n + c] : T(0);  // plain load: y may alias xin
          const T t = fma(a.c1, xown[c] - xp, xown[c]);
          out = fixd ? T(0) : fma(a.c2, (ldx(a.b + 3 * n + c) - Ax) / d, t);
        }
        a.y[3 * n + c] = out;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
  }

  if (MODE == OP_APPLY_DOT || MODE == OP_RESID_NORM) {
    double v[1] = {acc0};
    block_reduce_finalize<1>(a.red, v);
  }
}

template <typename T>
static ModalK<T> cast_modal(const ModalK<double>& K) {
  ModalK<T> o;
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c)
      for (int c2 = 0; c2 < 3; ++c2) o.B[q][c][c2] = (T)K.B[q][c][c2];
  for (int c = 0; c < 3; ++c) o.dd[c] = (T)K.dd[c];
  return o;
}

template <typename T>
constexpr int op_tyw() { return sizeof(T) == 8 ? 8 : 16; }

template <typename T>
dim3 op_grid(const Grid& g, int kchunk) {
  constexpr int TYW = op_tyw<T>();
  return dim3((g.NX + 30) / 31, (g.NY + TYW - 2) / (TYW - 1), (g.NZ + kchunk - 1) / kchunk);
}

template <typename T>
long long op_num_blocks(const Grid& g, int kchunk) {
  dim3 d = op_grid<T>(g, kchunk);
  return (long long)d.x * d.y * d.z;
}

template <typename T>
void launch_op(int mode, const OpArgs<T>& a, cudaStream_t st) {
  constexpr int TYW = op_tyw<T>();
  const dim3 grid = op_grid<T>(a.g, a.kchunk);
  const dim3 block(32, TYW);
  switch (mode) {
    case OP_APPLY: op_kernel<T, OP_APPLY, TYW><<<grid, block, 0, st>>>(a); break;
    case OP_APPLY_DOT: op_kernel<T, OP_APPLY_DOT, TYW><<<grid, block, 0, st>>>(a); break;
    case OP_RESID: op_kernel<T, OP_RESID, TYW><<<grid, block, 0, st>>>(a); break;
    case OP_RESID_NORM: op_kernel<T, OP_RESID_NORM, TYW><<<grid, block, 0, st>>>(a); break;
    case OP_JACOBI: op_kernel<T, OP_JACOBI, TYW><<<grid, block, 0, st>>>(a); break;
    case OP_CHEB2: op_kernel<T, OP_CHEB2, TYW><<<grid, block, 0, st>>>(a); break;
    default: break;
  }
}

template void launch_op<double>(int, const OpArgs<double>&, cudaStream_t);
template void launch_op<float>(int, const OpArgs<float>&, cudaStream_t);
template long long op_num_blocks<double>(const Grid&, int);
template long long op_num_blocks<float>(const Grid&, int);
template ModalK<float> cast_modal<float>(const ModalK<double>&);
template ModalK<double> cast_modal<double>(const ModalK<double>&);

ModalK<float> modal_to_f32(const ModalK<double>& K) { return cast_modal<float>(K); }

}  // namespace hexa
