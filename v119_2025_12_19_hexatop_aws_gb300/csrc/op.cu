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
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

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

// Addressing of one element column's four corner nodes (cc = dx + 2*dy):
// x/y validity is fixed per thread, each node layer adds one plane offset.
// A corner outside the grid is read at the nearest grid node (clamped index):
// every element that has such a corner lies outside the grid and has factor
// zero, so the (finite) value read never reaches a result, and the loads need
// no per-corner bounds test.
template <typename IX>
struct ColumnAddr {
  IX base;   // 3 * node index of corner 0 at layer 0
  IX row3;   // 3 * NX: corner 2 is one node row up
  IX plane3; // 3 * NX * NY
  IX off[4]; // 3 * (clamped) node index of each corner within a layer
};

template <typename IX>
__device__ __forceinline__ ColumnAddr<IX> column_addr(const Grid& g, int ie, int je) {
  ColumnAddr<IX> a;
  a.base = (IX)3 * ((IX)ie + (IX)g.NX * je);
  a.row3 = (IX)3 * g.NX;
  a.plane3 = (IX)3 * g.NX * g.NY;
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const int i = min(max(ie + (cc & 1), 0), g.NX - 1), j = min(max(je + (cc >> 1), 0), g.NY - 1);
    a.off[cc] = (IX)3 * ((IX)i + (IX)g.NX * j);
  }
  return a;
}

// Corner values of the column at node layer kk, read at clamped positions
// (see ColumnAddr).  INTERIOR: every corner of every column of the tile lies
// inside the grid in x and y; layers outside the grid read as zeros.
template <typename T, typename IX, bool INTERIOR = false>
__device__ __forceinline__ void load_corners(const Grid& g, const ColumnAddr<IX>& ca, const T* __restrict__ x, int kk,
                                             T (&v)[4][3]) {
  const bool kok = (kk >= 0) && (kk < g.NZ);
  const IX lb = ca.base + ca.plane3 * (IX)kk;
  if (INTERIOR) {
    if (kok) {
      const T* __restrict__ p0 = x + lb;
      const T* __restrict__ p2 = p0 + ca.row3;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[0][c] = ldx(p0 + c);
        v[1][c] = ldx(p0 + 3 + c);
        v[2][c] = ldx(p2 + c);
        v[3][c] = ldx(p2 + 3 + c);
      }
    } else {
#pragma unroll
      for (int cc = 0; cc < 4; ++cc)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[cc][c] = T(0);
    }
    return;
  }
  const IX L = ca.plane3 * (IX)min(max(kk, 0), g.NZ - 1);
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const T* __restrict__ p = x + (L + ca.off[cc]);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[cc][c] = ldx(p + c);
  }
}

// 1/d for the smoothers: correctly rounded in FP32; in FP64 a float seed and
// two Newton steps (relative error far below 1e-15).  Both are deterministic.
// The FP32 hardware approximation (rcp.approx, HEXA_OP_RCP_APPROX=1) measured
// slower in the Chebyshev step on the 384x192x192 grid (311 us against 251 us).
#ifndef HEXA_OP_RCP_APPROX
#define HEXA_OP_RCP_APPROX 0
#endif
__device__ __forceinline__ float recip(float d) {
#if HEXA_OP_RCP_APPROX
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
  return r;
#else
  return __frcp_rn(d);
#endif
}
__device__ __forceinline__ double recip(double d) {
  double r = (double)__frcp_rn((float)d);
  r = r * fma(-d, r, 2.0);
  r = r * fma(-d, r, 2.0);
  return r;
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

// FP32 forms with the (x, y) components packed in a float2, so that the
// butterflies and the z stage run as Blackwell's two-lane FP32 instructions
// (FADD2/FFMA2: one issue slot for two operations); z stays scalar.
#ifndef HEXA_OP_PACKED
#define HEXA_OP_PACKED 1
#endif
__device__ __forceinline__ float2 pk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

#if HEXA_OP_PACKED
template <>
__device__ __forceinline__ void xy_forward<float>(const float (&v)[4][3], float (&m)[4][3]) {
  const float2 v0 = pk(v[0][0], v[0][1]), v1 = pk(v[1][0], v[1][1]), v2 = pk(v[2][0], v[2][1]),
               v3 = pk(v[3][0], v[3][1]);
  const float2 a0 = pk_add(v0, v1), a1 = pk_sub(v1, v0), b0 = pk_add(v2, v3), b1 = pk_sub(v3, v2);
  const float2 m0 = pk_add(a0, b0), m1 = pk_add(a1, b1), m2 = pk_sub(b0, a0), m3 = pk_sub(b1, a1);
  m[0][0] = m0.x, m[0][1] = m0.y, m[1][0] = m1.x, m[1][1] = m1.y;
  m[2][0] = m2.x, m[2][1] = m2.y, m[3][0] = m3.x, m[3][1] = m3.y;
  const float a0z = v[0][2] + v[1][2], a1z = v[1][2] - v[0][2];
  const float b0z = v[2][2] + v[3][2], b1z = v[3][2] - v[2][2];
  m[0][2] = a0z + b0z, m[1][2] = a1z + b1z, m[2][2] = b0z - a0z, m[3][2] = b1z - a1z;
}

template <>
__device__ __forceinline__ void xy_inverse<float>(const float (&m)[4][3], float (&v)[4][3]) {
  const float2 m0 = pk(m[0][0], m[0][1]), m1 = pk(m[1][0], m[1][1]), m2 = pk(m[2][0], m[2][1]),
               m3 = pk(m[3][0], m[3][1]);
  const float2 A0 = pk_sub(m0, m2), B0 = pk_add(m0, m2), A1 = pk_sub(m1, m3), B1 = pk_add(m1, m3);
  const float2 v0 = pk_sub(A0, A1), v1 = pk_add(A0, A1), v2 = pk_sub(B0, B1), v3 = pk_add(B0, B1);
  v[0][0] = v0.x, v[0][1] = v0.y, v[1][0] = v1.x, v[1][1] = v1.y;
  v[2][0] = v2.x, v[2][1] = v2.y, v[3][0] = v3.x, v[3][1] = v3.y;
  const float A0z = m[0][2] - m[2][2], B0z = m[0][2] + m[2][2];
  const float A1z = m[1][2] - m[3][2], B1z = m[1][2] + m[3][2];
  v[0][2] = A0z - A1z, v[1][2] = A0z + A1z, v[2][2] = B0z - B1z, v[3][2] = B0z + B1z;
}
#endif

// lo += carry (the upper half of the element below)
template <typename T>
__device__ __forceinline__ void add_carry(T (&lo)[4][3], const T (&carry)[4][3]) {
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int c = 0; c < 3; ++c) lo[m][c] += carry[m][c];
}
#if HEXA_OP_PACKED
template <>
__device__ __forceinline__ void add_carry<float>(float (&lo)[4][3], const float (&carry)[4][3]) {
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const float2 t = pk_add(pk(lo[m][0], lo[m][1]), pk(carry[m][0], carry[m][1]));
    lo[m][0] = t.x, lo[m][1] = t.y;
    lo[m][2] += carry[m][2];
  }
}
#endif

// One element: lower/upper xy-modal node data -> lower/upper xy-modal
// contributions of f * K0 * u_e.
template <typename T>
__device__ __forceinline__ void element_modal(const ModalK<T>& K, const T (&L)[4][3],
                                              const T (&U)[4][3], T f, T (&lo)[4][3], T (&hi)[4][3]) {
  // z stage with the element factor folded in: f(L+U), f(U-L)
  T uh[8][3];
#pragma unroll
  for (int mxy = 0; mxy < 4; ++mxy)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T fu = f * U[mxy][c];
      uh[mxy][c] = fma(f, L[mxy][c], fu);
      uh[mxy + 4][c] = fma(-f, L[mxy][c], fu);
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
      wh[m][c] = s;
    }
#pragma unroll
  for (int mxy = 0; mxy < 4; ++mxy)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[mxy][c] = wh[mxy][c] - wh[mxy + 4][c];
      hi[mxy][c] = wh[mxy][c] + wh[mxy + 4][c];
    }
}

#if HEXA_OP_PACKED
template <>
__device__ __forceinline__ void element_modal<float>(const ModalK<float>& K, const float (&L)[4][3],
                                                     const float (&U)[4][3], float f, float (&lo)[4][3],
                                                     float (&hi)[4][3]) {
  const float2 f2 = pk(f, f), nf2 = pk(-f, -f);
  float uh[8][3];
#pragma unroll
  for (int mxy = 0; mxy < 4; ++mxy) {
    const float2 fu = __fmul2_rn(f2, pk(U[mxy][0], U[mxy][1]));
    const float2 l = pk(L[mxy][0], L[mxy][1]);
    const float2 s0 = __ffma2_rn(f2, l, fu), s1 = __ffma2_rn(nf2, l, fu);
    uh[mxy][0] = s0.x, uh[mxy][1] = s0.y, uh[mxy + 4][0] = s1.x, uh[mxy + 4][1] = s1.y;
    const float fuz = f * U[mxy][2];
    uh[mxy][2] = fmaf(f, L[mxy][2], fuz);
    uh[mxy + 4][2] = fmaf(-f, L[mxy][2], fuz);
  }
  float wh[8][3];
#pragma unroll
  for (int m = 0; m < 8; ++m)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int q = m ^ (1 << c);
      float s = 0.f;
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        if (modal_nz(q, c, c2)) s = fmaf(K.B[q][c][c2], uh[q ^ (1 << c2)][c2], s);
      wh[m][c] = s;
    }
#pragma unroll
  for (int mxy = 0; mxy < 4; ++mxy) {
    const float2 w0 = pk(wh[mxy][0], wh[mxy][1]), w1 = pk(wh[mxy + 4][0], wh[mxy + 4][1]);
    const float2 l = pk_sub(w0, w1), h = pk_add(w0, w1);
    lo[mxy][0] = l.x, lo[mxy][1] = l.y, hi[mxy][0] = h.x, hi[mxy][1] = h.y;
    lo[mxy][2] = wh[mxy][2] - wh[mxy + 4][2];
    hi[mxy][2] = wh[mxy][2] + wh[mxy + 4][2];
  }
}
#endif

// CTA height in warps.  FP32: 16 warps, one CTA per SM (127 registers); 8-warp
// CTAs two per SM measured 5 % slower on the 384x192x192 Chebyshev step
// (359 us against 340 us), the larger halo outweighing the shorter barriers.
#ifndef HEXA_OP_TYW32
#define HEXA_OP_TYW32 16
#endif

template <typename T>
constexpr int op_tyw() { return sizeof(T) == 8 ? 8 : HEXA_OP_TYW32; }
#ifndef HEXA_OP_MINCTAS32
#define HEXA_OP_MINCTAS32 (HEXA_OP_TYW32 <= 8 ? 2 : 1)
#endif
template <typename T>
constexpr int op_min_ctas() { return sizeof(T) == 8 ? 1 : HEXA_OP_MINCTAS32; }


// Four values of the y-exchange as one 16-byte shared-memory access per thread
// (float4; two 16-byte halves for double).
__device__ __forceinline__ void store4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void store4(double* p, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}
__device__ __forceinline__ void load4(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
}
__device__ __forceinline__ void load4(const double* p, double (&v)[4]) {
  const double2 t0 = reinterpret_cast<const double2*>(p)[0], t1 = reinterpret_cast<const double2*>(p)[1];
  v[0] = t0.x, v[1] = t0.y, v[2] = t1.x, v[3] = t1.y;
}

// One work item: the node columns of tile (tx, ty) for node layers [k0, k1).
// IX is the index type: int whenever 3 * nNodes fits, which halves the
// integer work of the address arithmetic.
// Named barrier b (1..15) between the two neighbouring warps wy = b - 1 and
// wy = b.  In a layer each warp first meets the warp below on its own index,
// then the warp above on the next one: the rendezvous form a chain from warp 0
// up, so every barrier completes, and a warp cannot reach a barrier instance
// of the next layer before both warps have left this layer's.  With the
// double-buffered slots, a slot is rewritten two layers later, after its
// reader has passed the next layer's rendezvous.
// HEXA_OP_PAIR_SYNC=0 builds the one-CTA-barrier form (measured slower on the
// 384x192x192 grid: Chebyshev step 0.240 ms against 0.226 ms, Jacobi step
// 0.205 against 0.199, apply with p.Ap 0.209 against 0.199, residual equal).
#ifndef HEXA_OP_PAIR_SYNC
#define HEXA_OP_PAIR_SYNC 1
#endif
__device__ __forceinline__ void pair_barrier(int b) { asm volatile("bar.sync %0, 64;" ::"r"(b) : "memory"); }

template <typename T, int MODE, int TYW, typename IX, typename A, bool INTERIOR = false>
__device__ __forceinline__ void op_item(const A& a, int tx, int ty, int chunk,
                                        T (&xch)[2][TYW][32][4],
                                        double& acc0, long long co) {
  // the _DOT forms of the smoothing steps also sum b.y
  constexpr int BM = MODE == OP_JACOBI_DOT ? OP_JACOBI : (MODE == OP_CHEB2_DOT ? OP_CHEB2 : MODE);
  constexpr bool DOTB = MODE == OP_JACOBI_DOT || MODE == OP_CHEB2_DOT;
  constexpr int NX_OWN = 31, NY_OWN = TYW - 1;
  constexpr bool NEED_F = (BM == OP_JACOBI || BM == OP_CHEB2);
  static_assert(TYW <= 16, "pairwise barriers use the named barriers 1..TYW-1");
  const Grid& g = a.g;
  const int lane = threadIdx.x, wy = threadIdx.y;
  const int i0 = tx * NX_OWN, j0 = ty * NY_OWN;
  const int k0 = chunk * a.kchunk;
  const int k1 = min(k0 + a.kchunk, g.NZ);
  const int ie = i0 - 1 + lane, je = j0 - 1 + wy;
  const bool colv = INTERIOR || ((ie >= 0) && (ie < g.nx) && (je >= 0) && (je < g.ny));
  const IX ecol = colv ? ((IX)ie + (IX)g.nx * je) : (IX)0;
  const IX eplane = (IX)g.nx * g.ny;
  const int in = i0 + lane, jn = j0 + wy;
  const bool own = (lane < NX_OWN) && (wy < NY_OWN) && (INTERIOR || ((in < g.NX) && (jn < g.NY)));
  // column co / ndof of a multi-column apply (the factors are shared)
  const T* __restrict__ x = a.x + co;
  const T* __restrict__ bv = a.b ? a.b + co : a.b;
  T* yv = a.y + co;  // not restrict: CHEB2 runs in place (xin == y)
  const T* xinv = a.xin ? a.xin + co : a.xin;
  const T* __restrict__ fac = a.fac;
  const ColumnAddr<IX> ca = column_addr<IX>(g, ie, je);
  // Dirichlet bits of this thread's node column: the x/y faces are fixed per
  // column, the z faces and the optional node mask are tested per layer
  const uint32_t F = a.m.faces;
  const unsigned colfix = (!INTERIOR && (((F & 1u) && in == 0) || ((F & 2u) && in == g.NX - 1) ||
                                          ((F & 4u) && jn == 0) || ((F & 8u) && jn == g.NY - 1))) ? 7u : 0u;
  const IX nplane = (IX)g.NX * g.NY;
  const IX ncol = (IX)in + (IX)g.NX * jn;

  auto facload = [&](int k) -> T {
    return (colv && k >= 0 && k < g.nz) ? ldx(fac + ecol + eplane * k) : T(0);
  };
  T Lm[4][3], carry[4][3], xown[3];
  T fprev;
  {
    T raw[4][3];
    load_corners<T, IX, INTERIOR>(g, ca, x, k0 - 1, raw);
    T Lprev[4][3];
    xy_forward<T>(raw, Lprev);
    load_corners<T, IX, INTERIOR>(g, ca, x, k0, raw);
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
    xy_forward<T>(raw, Lm);
    fprev = facload(k0 - 1);
    T lo[4][3];
    element_modal<T>(a.K, Lprev, Lm, fprev, lo, carry);
  }
  // b and the previous iterate at the own node are loaded one layer ahead, so
  // their DRAM latency hides behind the next layer's element work
  constexpr bool NEED_B = BM == OP_RESID || BM == OP_RESID_NORM || BM == OP_JACOBI || BM == OP_CHEB2;
  constexpr bool NEED_P = BM == OP_CHEB2;
  T bnext[3] = {T(0), T(0), T(0)}, pnext[3] = {T(0), T(0), T(0)};
  auto load_bp = [&](int kk) {
    if (own) {
      const IX n3 = (IX)3 * (ncol + nplane * (IX)kk);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (NEED_B) bnext[c] = ldx(bv + n3 + c);
        if (NEED_P) pnext[c] = xinv ? xinv[n3 + c] : T(0);  // plain load: y may alias xin
      }
    }
  };
  if (NEED_B || NEED_P) load_bp(k0);

  // sums of this item in the kernel's own precision (one item is at most a
  // few dozen layers per thread), folded into the FP64 accumulator at the end:
  // FP64 arithmetic in the FP32 kernels would run at GB300's FP64 rate
  T accT = T(0);
  T nraw[4][3];
  load_corners<T, IX, INTERIOR>(g, ca, x, k0 + 1, nraw);
  T fnext = facload(k0);

  // three layers per unrolled step for the Chebyshev forms, two for the rest
  // (on the 384x192x192 grid: Chebyshev step 0.2191 ms at 3 against 0.2248
  // at 2 and 0.2475 at 1; Jacobi step 0.2006 at 3, 0.1983 at 2)
#pragma unroll(BM == OP_CHEB2 ? 3 : 2)
  for (int k = k0; k < k1; ++k) {
    T raw[4][3];
#pragma unroll
    for (int cc = 0; cc < 4; ++cc)
#pragma unroll
      for (int c = 0; c < 3; ++c) raw[cc][c] = nraw[cc][c];
    const T f = fnext;
    T bk[3], pk3[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) bk[c] = bnext[c], pk3[c] = pnext[c];
    if (k + 1 < k1) {  // prefetch the next layer
      load_corners<T, IX, INTERIOR>(g, ca, x, k + 2, nraw);
      fnext = facload(k + 1);
      if (NEED_B || NEED_P) load_bp(k + 1);
    }
    T Um[4][3];
    xy_forward<T>(raw, Um);
    T lo[4][3], hi[4][3];
    element_modal<T>(a.K, Lm, Um, f, lo, hi);
    add_carry<T>(lo, carry);
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
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
    store4(&xch[buf][wy][lane][0], T0[0], T0[1], T0[2], F1);  // one vector store, no bank conflicts
#if HEXA_OP_PAIR_SYNC
    // warp wy reads only what warp wy + 1 stored: rendezvous with the warp
    // below (which reads this warp's slot), then with the warp above
    if (wy >= 1) pair_barrier(wy);
    if (wy + 1 < TYW) pair_barrier(wy + 1);
#else
    __syncthreads();
#endif
    if (own) {
      const IX n = ncol + nplane * (IX)k;
      unsigned fx = colfix;
      if (((F & 16u) && k == 0) || ((F & 32u) && k == g.NZ - 1)) fx = 7u;
      if (a.m.node) fx |= (unsigned)__ldg(a.m.node + n);
      T nb[4];
      load4(&xch[buf][wy + 1][lane][0], nb);
      T Kx[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) Kx[c] = T1[c] + nb[c];
      T dinv[3] = {T(0), T(0), T(0)};
      if (NEED_F) {
        const T fsum = F1 + nb[3];
        if (a.diag_quirk) {
          const T r = recip(fma(a.K.dd[0], fsum, a.sigma));
          dinv[0] = dinv[1] = dinv[2] = r;
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c) dinv[c] = recip(fma(a.K.dd[c], fsum, a.sigma));
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const bool fixd = (fx >> c) & 1u;
        const T Ax = fma(a.sigma, xown[c], Kx[c]);
        T out;
        if (BM == OP_APPLY) {
          out = fixd ? T(0) : Ax;
        } else if (BM == OP_APPLY_DOT) {
          out = fixd ? T(0) : Ax;
          accT = fma(xown[c], out, accT);
        } else if (BM == OP_RESID || BM == OP_RESID_NORM) {
          out = fixd ? T(0) : (bk[c] - Ax);
          if (BM == OP_RESID_NORM) accT = fma(out, out, accT);
        } else if (BM == OP_JACOBI) {  // x + omega (b - Ax) / D
          out = fixd ? T(0) : fma(a.omega * dinv[c], bk[c] - Ax, xown[c]);
        } else {  // OP_CHEB2: x + c1 (x - x_prev) + c2 D^-1 (b - Ax)
          const T t = fma(a.c1, xown[c] - pk3[c], xown[c]);
          out = fixd ? T(0) : fma(a.c2 * dinv[c], bk[c] - Ax, t);
        }
        if (DOTB) accT = fma(bk[c], out, accT);
        yv[3 * n + c] = out;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
  }

  acc0 += (double)accT;
  __syncthreads();  // the next item reuses xch
}

// Whether every corner of every column of tile (tx, ty) lies inside the grid
// in x and y (the predicate-free form of the item applies).  Off by default:
// with both item forms inlined the kernels spill, and on the 384x192x192 grid
// the residual gained 6 % while the plain apply lost 18 %.
#ifndef HEXA_OP_INTERIOR
#define HEXA_OP_INTERIOR 0
#endif
template <int TYW>
__device__ __forceinline__ bool tile_interior(const Grid& g, int tx, int ty) {
  const int i0 = tx * 31, j0 = ty * (TYW - 1);
  return i0 >= 1 && i0 + 31 <= g.NX - 1 && j0 >= 1 && j0 + TYW - 1 <= g.NY - 1;
}

template <typename T, int MODE, int TYW, typename IX, bool MULTI>
__global__ void __launch_bounds__(32 * TYW, op_min_ctas<T>()) op_kernel(const OpArgs<T> a) {
  if (a.halt && *((volatile const int*)a.halt)) return;
  __shared__ __align__(16) T xch[2][TYW][32][4];
  double acc0 = 0.0;
  // static stride over (tile x, tile y, z-chunk) items: deterministic, and
  // with the grid sized to the resident CTAs no wave is left half empty
  const int nxy = a.tiles_x * a.tiles_y;
  const int items = nxy * a.nchunks;
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int chunk = item / nxy, t = item - chunk * nxy;
    const int ty = t / a.tiles_x, tx = t - ty * a.tiles_x;
    if (MULTI) {  // every column of a multi-column apply reuses the item's factors from L1
      for (int col = 0; col < a.ncol; ++col) op_item<T, MODE, TYW, IX>(a, tx, ty, chunk, xch, acc0, col * a.g.ndof());
    } else if (HEXA_OP_INTERIOR && tile_interior<TYW>(a.g, tx, ty)) {
      op_item<T, MODE, TYW, IX, OpArgs<T>, true>(a, tx, ty, chunk, xch, acc0, 0);
    } else {
      op_item<T, MODE, TYW, IX>(a, tx, ty, chunk, xch, acc0, 0);
    }
  }
  if (MODE == OP_APPLY_DOT || MODE == OP_RESID_NORM || MODE == OP_JACOBI_DOT || MODE == OP_CHEB2_DOT) {
    double v[1] = {acc0};
    block_reduce_finalize<1>(a.red, v);
  }
}

// ------------------------------------------------- TMA-staged FP32 operator
// The same node-centric product with the new node layer of x staged in shared
// memory by the TMA engine instead of twelve predicated global loads per
// thread and layer: for each layer a CTA needs, one thread per node row of
// the tile (lane 0 of warp r for row r, lane 1 of warp 0 for the last row, so
// that no warp carries the issue work of the others into the per-layer
// barrier) issues one bulk copy (cp.async.bulk) of that row's 33 nodes into a
// ring of NS layer slots and arrives on the slot's mbarrier with the copy's
// transaction bytes.  Threads read their four corners with plain shared-memory loads at
// fixed offsets: no address arithmetic and no bounds tests per corner.
// Rows and layers outside the grid are not copied; the only elements that
// read them have factor zero (element column, row or layer outside the grid),
// so stale slot contents never reach a result (the ring is zeroed at start so
// that they are finite).  Rows start at any 4-byte offset while bulk copies
// move whole 16-byte granules: each copy is widened to the granules around
// the row (never past a granule that holds some of the row, so it stays inside
// x's allocation) and lands so that the row's first node sits aoff floats into
// its slot; the producer lane records aoff beside the data.  The ring keeps
// NS layers in flight across the CTA's whole sequence of work items, so
// items do not drain the pipeline.  Every wait is bounded (about half a
// second of clock cycles): a wait that runs out sets the device error word
// g_op_wait_err, every thread of the CTA leaves at the next barrier, the
// copies still in flight are waited for (bounded again) and the kernel
// returns; the host reads the word after the call (op_wait_error).
namespace tma {
constexpr int NS = 4;        // layer slots in flight
constexpr int PITCH = 112;   // floats per staged node row: 33 nodes x 3 + granule slack
constexpr long long kWaitCycles = 1000000000LL;
}  // namespace tma

__device__ int g_op_wait_err = 0;

template <int TYW>
struct OpRing {
  float v[tma::NS][TYW + 1][tma::PITCH];
  int aoff[tma::NS][TYW + 1];
  unsigned long long bar[tma::NS];
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, uint32_t bytes) {
  asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }" ::"r"(smem_addr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("{ .reg .b64 st; mbarrier.arrive.shared::cta.b64 st, [%0]; }" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, uint32_t parity) {
  uint32_t ok;
  asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
               : "=r"(ok)
               : "r"(smem_addr(b)), "r"(parity)
               : "memory");
  return ok != 0;
}
// bounded: false when the slot did not fill within tma::kWaitCycles
__device__ __forceinline__ bool ring_wait(unsigned long long* b, uint32_t parity) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  do {
    if (mbar_try_wait(b, parity)) return true;
  } while (clock64() - t0 < tma::kWaitCycles);
  return false;
}

// The CTA's sequence of layer loads: item by item (static stride), node
// layers k0-1 .. k1 of each item's z-chunk.
struct LoadCursor {
  int item, kk, k1, tx, ty;
};
template <typename A>
__device__ __forceinline__ void cursor_start(const A& a, int item, LoadCursor& c) {
  const int nxy = a.tiles_x * a.tiles_y;
  const int chunk = item / nxy, t = item - chunk * nxy;
  c.item = item;
  c.ty = t / a.tiles_x;
  c.tx = t - c.ty * a.tiles_x;
  const int k0 = chunk * a.kchunk;
  c.kk = k0 - 1;
  c.k1 = min(k0 + a.kchunk, a.g.NZ);
}

// Node row `row` of layer c.kk into slot q % NS, by the row's issuing thread:
// it arrives on the slot's mbarrier with the copy's bytes (a row outside the
// grid: a plain arrival).  test_stall: the load is left out, no arrival (a
// wait that runs out).
template <int TYW>
__device__ __forceinline__ void issue_row(OpRing<TYW>& R, int q, const Grid& g, const float* x, const LoadCursor& c,
                                          int row, bool test_stall) {
  if (test_stall) return;
  const int slot = q % tma::NS;
  unsigned long long* bar = &R.bar[slot];
  const int j = c.ty * (TYW - 1) - 1 + row;
  const int i0m = c.tx * 31 - 1;
  const int ifirst = max(i0m, 0), ilast = min(i0m + 32, g.NX - 1);
  if (j >= 0 && j < g.NY && c.kk >= 0 && c.kk < g.NZ) {
    const long long s = 3LL * ((long long)ifirst + (long long)g.NX * ((long long)j + (long long)g.NY * c.kk));
    const unsigned long long sb = (unsigned long long)(x + s);
    const unsigned long long b0 = sb & ~15ull;
    const unsigned long long b1 = (sb + 12ull * (unsigned long long)(ilast - ifirst + 1) + 15ull) & ~15ull;
    const int slack = (int)((sb & 15ull) >> 2), delta = ifirst - i0m;
    const int aoff = (slack - 3 * delta) & 3;
    float* dst = &R.v[slot][row][aoff + 3 * delta - slack];  // 0 or 4 floats in: 16-byte aligned
    const uint32_t bytes = (uint32_t)(b1 - b0);
    R.aoff[slot][row] = aoff;
    mbar_arrive_expect_tx(bar, bytes);
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(b0), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
  } else {
    R.aoff[slot][row] = 0;
    mbar_arrive(bar);
  }
}

// The issuing thread of each row: lane 0 of warp r for rows 0..TYW-1, lane 1
// of warp 0 for row TYW; -1 for every other thread.
template <int TYW>
__device__ __forceinline__ int my_row() {
  return threadIdx.x == 0 ? (int)threadIdx.y : ((threadIdx.x == 1 && threadIdx.y == 0) ? TYW : -1);
}

// Issue loads while fewer than NS are outstanding; every thread walks the
// cursor (uniform integer work), the row owners issue.
template <int TYW, typename A>
__device__ __forceinline__ void produce_loads(const A& a, OpRing<TYW>& R, int cq, int& pq, LoadCursor& pc,
                                              int& p_items_left) {
  const int row = my_row<TYW>();
  const bool stall_cta = a.test_stall >= 0 && blockIdx.x == 0;
  while (p_items_left > 0 && pq < cq + tma::NS) {
    if (row >= 0) issue_row<TYW>(R, pq, a.g, a.x, pc, row, stall_cta && pq == a.test_stall);
    ++pq;
    if (++pc.kk > pc.k1) {
      if (--p_items_left > 0) cursor_start(a, pc.item + gridDim.x, pc);
    }
  }
}

template <int MODE, int TYW, typename IX>
__device__ __forceinline__ bool op_item_tma(const OpArgs<float>& a, const LoadCursor& it, OpRing<TYW>& R, int& cq,
                                            int& pq, LoadCursor& pc, int& p_items_left, float (&xch)[2][TYW][32][4],
                                            double& acc0) {
  using T = float;
  constexpr int BM = MODE == OP_JACOBI_DOT ? OP_JACOBI : (MODE == OP_CHEB2_DOT ? OP_CHEB2 : MODE);
  constexpr bool DOTB = MODE == OP_JACOBI_DOT || MODE == OP_CHEB2_DOT;
  constexpr int NX_OWN = 31, NY_OWN = TYW - 1;
  constexpr bool NEED_F = (BM == OP_JACOBI || BM == OP_CHEB2);
  const Grid& g = a.g;
  const int lane = threadIdx.x, wy = threadIdx.y;
  const int i0 = it.tx * NX_OWN, j0 = it.ty * NY_OWN;
  const int k0 = it.kk + 1, k1 = it.k1;
  const int ie = i0 - 1 + lane, je = j0 - 1 + wy;
  const bool colv = (ie >= 0) && (ie < g.nx) && (je >= 0) && (je < g.ny);
  const IX ecol = colv ? ((IX)ie + (IX)g.nx * je) : (IX)0;
  const IX eplane = (IX)g.nx * g.ny;
  const int in = i0 + lane, jn = j0 + wy;
  const bool own = (lane < NX_OWN) && (wy < NY_OWN) && (in < g.NX) && (jn < g.NY);
  const T* __restrict__ bv = a.b;
  T* yv = a.y;  // not restrict: CHEB2 runs in place (xin == y)
  const T* xinv = a.xin;
  const T* __restrict__ fac = a.fac;
  const uint32_t F = a.m.faces;
  const unsigned colfix =
      (((F & 1u) && in == 0) || ((F & 2u) && in == g.NX - 1) || ((F & 4u) && jn == 0) || ((F & 8u) && jn == g.NY - 1))
          ? 7u : 0u;
  const IX nplane = (IX)g.NX * g.NY;
  const IX ncol = (IX)in + (IX)g.NX * jn;
  bool bad = false;

  auto facload = [&](int k) -> T { return (colv && k >= 0 && k < g.nz) ? __ldg(fac + ecol + eplane * k) : T(0); };
  // the four corners of this thread's element column at the next staged layer
  auto take = [&](T (&v)[4][3]) {
    const int slot = cq % tma::NS;
    if (!ring_wait(&R.bar[slot], (uint32_t)((cq / tma::NS) & 1))) bad = true;
    const float* r0 = &R.v[slot][wy][R.aoff[slot][wy] + 3 * lane];
    const float* r1 = &R.v[slot][wy + 1][R.aoff[slot][wy + 1] + 3 * lane];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[0][c] = r0[c];
      v[1][c] = r0[3 + c];
      v[2][c] = r1[c];
      v[3][c] = r1[3 + c];
    }
    ++cq;
  };

  T Lm[4][3], carry[4][3], xown[3];
  T fprev;
  {
    T raw[4][3], Lprev[4][3], lo[4][3];
    take(raw);
    xy_forward<T>(raw, Lprev);
    take(raw);
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
    xy_forward<T>(raw, Lm);
    fprev = facload(k0 - 1);
    element_modal<T>(a.K, Lprev, Lm, fprev, lo, carry);
  }
  constexpr bool NEED_B = BM == OP_RESID || BM == OP_RESID_NORM || BM == OP_JACOBI || BM == OP_CHEB2;
  constexpr bool NEED_P = BM == OP_CHEB2;
  T bnext[3] = {T(0), T(0), T(0)}, pnext[3] = {T(0), T(0), T(0)};
  auto load_bp = [&](int kk) {
    if (own) {
      const IX n3 = (IX)3 * (ncol + nplane * (IX)kk);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (NEED_B) bnext[c] = __ldg(bv + n3 + c);
        if (NEED_P) pnext[c] = xinv ? xinv[n3 + c] : T(0);  // plain load: y may alias xin
      }
    }
  };
  if (NEED_B || NEED_P) load_bp(k0);
  T accT = T(0);
  T fnext = facload(k0);
  bool aborted = false;

#pragma unroll 2
  for (int k = k0; k < k1; ++k) {
    T raw[4][3];
    take(raw);
    const T f = fnext;
    T bk[3], pk3[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) bk[c] = bnext[c], pk3[c] = pnext[c];
    if (k + 1 < k1) {
      fnext = facload(k + 1);
      if (NEED_B || NEED_P) load_bp(k + 1);
    }
    T Um[4][3];
    xy_forward<T>(raw, Um);
    T lo[4][3], hi[4][3];
    element_modal<T>(a.K, Lm, Um, f, lo, hi);
    add_carry<T>(lo, carry);
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        carry[m][c] = hi[m][c];
        Lm[m][c] = Um[m][c];
      }
    T cv[4][3];
    xy_inverse<T>(lo, cv);
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
    store4(&xch[buf][wy][lane][0], T0[0], T0[1], T0[2], F1);
    if (__syncthreads_or(bad ? 1 : 0)) {  // a staging wait ran out somewhere in the CTA
      aborted = true;
      break;
    }
    produce_loads<TYW>(a, R, cq, pq, pc, p_items_left);  // every consumer has read the loads < cq
    if (own) {
      const IX n = ncol + nplane * (IX)k;
      unsigned fx = colfix;
      if (((F & 16u) && k == 0) || ((F & 32u) && k == g.NZ - 1)) fx = 7u;
      if (a.m.node) fx |= (unsigned)__ldg(a.m.node + n);
      T nb[4];
      load4(&xch[buf][wy + 1][lane][0], nb);
      T Kx[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) Kx[c] = T1[c] + nb[c];
      T dinv[3] = {T(0), T(0), T(0)};
      if (NEED_F) {
        const T fsum = F1 + nb[3];
        if (a.diag_quirk) {
          const T r = recip(fma(a.K.dd[0], fsum, a.sigma));
          dinv[0] = dinv[1] = dinv[2] = r;
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c) dinv[c] = recip(fma(a.K.dd[c], fsum, a.sigma));
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const bool fixd = (fx >> c) & 1u;
        const T Ax = fma(a.sigma, xown[c], Kx[c]);
        T out;
        if (BM == OP_APPLY) {
          out = fixd ? T(0) : Ax;
        } else if (BM == OP_APPLY_DOT) {
          out = fixd ? T(0) : Ax;
          accT = fma(xown[c], out, accT);
        } else if (BM == OP_RESID || BM == OP_RESID_NORM) {
          out = fixd ? T(0) : (bk[c] - Ax);
          if (BM == OP_RESID_NORM) accT = fma(out, out, accT);
        } else if (BM == OP_JACOBI) {
          out = fixd ? T(0) : fma(a.omega * dinv[c], bk[c] - Ax, xown[c]);
        } else {
          const T t = fma(a.c1, xown[c] - pk3[c], xown[c]);
          out = fixd ? T(0) : fma(a.c2 * dinv[c], bk[c] - Ax, t);
        }
        if (DOTB) accT = fma(bk[c], out, accT);
        yv[3 * n + c] = out;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
  }
  acc0 += (double)accT;
  if (aborted) return false;
  __syncthreads();  // the next item reuses xch
  return true;
}

template <int MODE, int TYW, typename IX>
__global__ void __launch_bounds__(32 * TYW, 1) op_tma_kernel(const OpArgs<float> a) {
  if (a.halt && *((volatile const int*)a.halt)) return;
  __shared__ __align__(16) float xch[2][TYW][32][4];
  __shared__ __align__(128) OpRing<TYW> R;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  {  // finite stale contents, then the barriers
    float* z = &R.v[0][0][0];
    for (int e = tid; e < tma::NS * (TYW + 1) * tma::PITCH; e += 32 * TYW) z[e] = 0.f;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) {
      for (int q = 0; q < tma::NS; ++q) mbar_init(&R.bar[q], TYW + 1);  // one arrival per node row
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
  }
  __syncthreads();
  const int nxy = a.tiles_x * a.tiles_y;
  const int items = nxy * a.nchunks;
  int p_items_left = items > (int)blockIdx.x ? (items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  int cq = 0, pq = 0;
  LoadCursor pc;
  if (p_items_left > 0) cursor_start(a, blockIdx.x, pc);
  produce_loads<TYW>(a, R, cq, pq, pc, p_items_left);  // prime the ring
  double acc0 = 0.0;
  bool ok = true;
  for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
    LoadCursor it;
    cursor_start(a, item, it);
    ok = op_item_tma<MODE, TYW, IX>(a, it, R, cq, pq, pc, p_items_left, xch, acc0);
  }
  if (!ok) {  // bounded drain of the copies still in flight, then report
    if (tid == 0) {
      for (int q = cq > 0 ? cq - 1 : 0; q < pq; ++q) ring_wait(&R.bar[q % tma::NS], (uint32_t)((q / tma::NS) & 1));
      atomicExch(&g_op_wait_err, 1);
    }
    __syncthreads();
  }
  if (MODE == OP_APPLY_DOT || MODE == OP_RESID_NORM || MODE == OP_JACOBI_DOT || MODE == OP_CHEB2_DOT) {
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


template <typename T, int MODE>
static int op_resident_ctas() {
  static int cached = 0;
  if (!cached) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, op_kernel<T, MODE, op_tyw<T>(), long long, false>,
                                                  32 * op_tyw<T>(), 0);
    cached = std::max(1, sms) * std::max(1, occ);
  }
  return cached;
}

template <typename T>
static int resident_ctas(int mode) {
  switch (mode) {
    case OP_APPLY: return op_resident_ctas<T, OP_APPLY>();
    case OP_APPLY_DOT: return op_resident_ctas<T, OP_APPLY_DOT>();
    case OP_RESID: return op_resident_ctas<T, OP_RESID>();
    case OP_RESID_NORM: return op_resident_ctas<T, OP_RESID_NORM>();
    case OP_JACOBI: return op_resident_ctas<T, OP_JACOBI>();
    default: return op_resident_ctas<T, OP_CHEB2>();
  }
}

template <typename T>
void op_tiles(const Grid& g, int kchunk, int* tx, int* ty, int* nch) {
  constexpr int TYW = op_tyw<T>();
  *tx = (g.NX + 30) / 31;
  *ty = (g.NY + TYW - 2) / (TYW - 1);
  *nch = (g.NZ + kchunk - 1) / kchunk;
}

// Largest CTA count any mode launches for this grid (sizes reduction partials).
template <typename T>
long long op_num_blocks(const Grid& g, int kchunk) {
  int tx, ty, nch;
  op_tiles<T>(g, kchunk, &tx, &ty, &nch);
  return (long long)tx * ty * nch;
}

template <typename T>
int op_pick_kchunk(const Grid& g) {
  int tx, ty, nch;
  op_tiles<T>(g, 1, &tx, &ty, &nch);
  const long long tiles = (long long)tx * ty;
  const long long want = 8LL * resident_ctas<T>(OP_CHEB2);  // ~8 items per CTA
  long long chunks = (want + tiles - 1) / tiles;
  chunks = std::max<long long>(1, std::min<long long>(chunks, (g.NZ + 15) / 16));  // chunks of >= 16 layers
  return (int)((g.NZ + chunks - 1) / chunks);
}

static int env_int(const char* name, int dflt) {
  const char* v = std::getenv(name);
  return (v && *v) ? std::atoi(v) : dflt;
}

// Form of FP32 single-column launches (HEXA_OP_FORM, read once): 0 (default)
// the one-row kernel with per-thread global loads, 1 the TMA-staged kernel
// (measured slower on GB300: more instructions in an issue-bound kernel);
// HEXA_OP_TEST_STALL=q makes CTA 0 of the TMA-staged kernel leave out its
// layer load q (tests of the bounded waits).
static int op_form() {
  static const int form = env_int("HEXA_OP_FORM", 0);
  return form;
}

static int tma_resident_ctas() {
  static int cached = 0;
  if (!cached) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, op_tma_kernel<OP_CHEB2, HEXA_OP_TYW32, int>, 32 * HEXA_OP_TYW32,
                                                  0);
    cached = std::max(1, sms) * std::max(1, occ);
  }
  return cached;
}

bool op_take_wait_error(cudaStream_t st) {
  int h = 0;
  if (cudaMemcpyFromSymbolAsync(&h, g_op_wait_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (h) {
    static const int zero = 0;
    cudaMemcpyToSymbolAsync(g_op_wait_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  return h != 0;
}

static void launch_op_tma(int mode, OpArgs<float>& a, bool i32, cudaStream_t st) {
  constexpr int TYW = HEXA_OP_TYW32;
  static const int stall = env_int("HEXA_OP_TEST_STALL", -1);
  a.test_stall = stall;
  const long long items = (long long)a.tiles_x * a.tiles_y * a.nchunks;
  const int grid = (int)std::min<long long>(items, tma_resident_ctas());
  const dim3 block(32, TYW);
#define HEXA_OPT_CASE(M)                                                          \
  case M:                                                                        \
    if (i32) op_tma_kernel<M, TYW, int><<<grid, block, 0, st>>>(a);              \
    else op_tma_kernel<M, TYW, long long><<<grid, block, 0, st>>>(a);            \
    break;
  switch (mode) {
    HEXA_OPT_CASE(OP_APPLY)
    HEXA_OPT_CASE(OP_APPLY_DOT)
    HEXA_OPT_CASE(OP_RESID)
    HEXA_OPT_CASE(OP_RESID_NORM)
    HEXA_OPT_CASE(OP_JACOBI)
    HEXA_OPT_CASE(OP_CHEB2)
    HEXA_OPT_CASE(OP_JACOBI_DOT)
    HEXA_OPT_CASE(OP_CHEB2_DOT)
    default: break;
  }
#undef HEXA_OPT_CASE
}

template <typename T>
void launch_op(int mode, const OpArgs<T>& a0, cudaStream_t st) {
  constexpr int TYW = op_tyw<T>();
  OpArgs<T> a = a0;
  op_tiles<T>(a.g, a.kchunk, &a.tiles_x, &a.tiles_y, &a.nchunks);
  const long long items = (long long)a.tiles_x * a.tiles_y * a.nchunks;
  const int grid = (int)std::min<long long>(items, resident_ctas<T>(mode));
  const dim3 block(32, TYW);
  const bool i32 = a.g.ndof() < (1LL << 30) && a.g.nelem() < (1LL << 30);
  if constexpr (sizeof(T) == 4) {
    if (a.ncol <= 1 && op_form() == 1) {
      launch_op_tma(mode, a, i32, st);
      return;
    }
  }
  if (a.ncol > 1) {  // multi-column forms (no reductions): apply, residual and the two smoothing steps
    if (mode == OP_APPLY) {
      if (i32) op_kernel<T, OP_APPLY, TYW, int, true><<<grid, block, 0, st>>>(a);
      else op_kernel<T, OP_APPLY, TYW, long long, true><<<grid, block, 0, st>>>(a);
    } else if (mode == OP_RESID) {
      if (i32) op_kernel<T, OP_RESID, TYW, int, true><<<grid, block, 0, st>>>(a);
      else op_kernel<T, OP_RESID, TYW, long long, true><<<grid, block, 0, st>>>(a);
    } else if (mode == OP_JACOBI) {
      if (i32) op_kernel<T, OP_JACOBI, TYW, int, true><<<grid, block, 0, st>>>(a);
      else op_kernel<T, OP_JACOBI, TYW, long long, true><<<grid, block, 0, st>>>(a);
    } else if (mode == OP_CHEB2) {
      if (i32) op_kernel<T, OP_CHEB2, TYW, int, true><<<grid, block, 0, st>>>(a);
      else op_kernel<T, OP_CHEB2, TYW, long long, true><<<grid, block, 0, st>>>(a);
    }
    return;
  }
#define HEXA_OP_CASE(M)                                                              \
  case M:                                                                           \
    if (i32) op_kernel<T, M, TYW, int, false><<<grid, block, 0, st>>>(a);           \
    else op_kernel<T, M, TYW, long long, false><<<grid, block, 0, st>>>(a);         \
    break;
  switch (mode) {
    HEXA_OP_CASE(OP_APPLY)
    HEXA_OP_CASE(OP_APPLY_DOT)
    HEXA_OP_CASE(OP_RESID)
    HEXA_OP_CASE(OP_RESID_NORM)
    HEXA_OP_CASE(OP_JACOBI)
    HEXA_OP_CASE(OP_CHEB2)
    HEXA_OP_CASE(OP_JACOBI_DOT)
    HEXA_OP_CASE(OP_CHEB2_DOT)
    default: break;
  }
#undef HEXA_OP_CASE
}

// ---------------------------------------------------------------- batches
// The arguments op_item reads, for one instance of a batch: the grid, the
// mask and the pointers of the instance, the shared K0 blocks by reference
// (to the kernel's __grid_constant__ parameter: no copy).
template <typename T>
struct ItemArgs {
  Grid g;
  Mask m;
  const T* x;
  const T* fac;
  const T* b;
  T* y;
  const T* xin;
  T c1, c2;
  const ModalK<T>& K;
  T sigma, omega;
  int kchunk, diag_quirk;
};

__device__ __forceinline__ int batch_find_op(const BatchInst* in, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (in[mid].oblk0 <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One launch over every instance of a batch: instance i's blocks run the
// static-stride item loop of op_kernel over its own (tile, z-chunk) items;
// an instance whose solve has halted returns at once.
template <typename T, int MODE, int TYW, typename IX>
__global__ void __launch_bounds__(32 * TYW, op_min_ctas<T>()) op_batch_kernel(const __grid_constant__ BatchOpArgs<T> a) {
  __shared__ __align__(16) T xch[2][TYW][32][4];
  const BatchInst& I = a.inst[batch_find_op(a.inst, a.ninst, blockIdx.x)];
  const int id = I.id;
  if (a.s && *((volatile const int*)&a.s[id].halt)) return;
  const ItemArgs<T> ia{I.g,      I.m,      a.x + I.off,  a.fac + I.eoff,  a.b ? a.b + I.off : a.b,
                       a.y + I.off, a.xin ? a.xin + I.off : a.xin, a.c1, a.c2, a.K, (T)I.sigma, a.omega,
                       I.kchunk, a.diag_quirk};
  const int txs = I.tiles_x, nxy = I.tiles_x * I.tiles_y, items = nxy * I.nchunks;
  const int local = blockIdx.x - I.oblk0, nb = I.onblk;
  double acc0 = 0.0;
  for (int item = local; item < items; item += nb) {
    const int chunk = item / nxy, t = item - chunk * nxy;
    const int ty = t / txs, tx = t - ty * txs;
    op_item<T, MODE, TYW, IX>(ia, tx, ty, chunk, xch, acc0, 0);
  }
  if (MODE == OP_APPLY_DOT || MODE == OP_RESID_NORM) {
    double v[1] = {acc0};
    block_reduce_finalize_at<1>(a.red, v, id, blockIdx.x, nb, I.oblk0, 1);
  }
}

template <typename T>
int op_batch_plan(BatchInst* in, int n, int kchunk) {
  long long total = 0;
  std::vector<long long> items(n);
  const int kc = kchunk > 0 ? kchunk : 16;
  for (int i = 0; i < n; ++i) {
    BatchInst& b = in[i];
    b.kchunk = std::max(1, std::min(kc, b.g.NZ));
    op_tiles<T>(b.g, b.kchunk, &b.tiles_x, &b.tiles_y, &b.nchunks);
    items[i] = (long long)b.tiles_x * b.tiles_y * b.nchunks;
    total += items[i];
  }
  const double per = std::max(1.0, (double)total / std::max(1, resident_ctas<T>(OP_CHEB2)));
  int blk = 0;
  for (int i = 0; i < n; ++i) {
    const long long want = (long long)std::ceil((double)items[i] / per);
    in[i].oblk0 = blk;
    in[i].onblk = (int)std::max<long long>(1, std::min<long long>(items[i], want));
    blk += in[i].onblk;
  }
  return blk;
}

template <typename T>
void launch_op_batch(int mode, const BatchOpArgs<T>& a0, bool idx32, cudaStream_t st) {
  constexpr int TYW = op_tyw<T>();
  const dim3 block(32, TYW);
  const BatchOpArgs<T>& a = a0;
#define HEXA_OPB_CASE(M)                                                                          \
  case M:                                                                                        \
    if (idx32) op_batch_kernel<T, M, TYW, int><<<a.nblocks, block, 0, st>>>(a);                  \
    else op_batch_kernel<T, M, TYW, long long><<<a.nblocks, block, 0, st>>>(a);                  \
    break;
  switch (mode) {
    HEXA_OPB_CASE(OP_APPLY)
    HEXA_OPB_CASE(OP_APPLY_DOT)
    HEXA_OPB_CASE(OP_RESID)
    HEXA_OPB_CASE(OP_RESID_NORM)
    HEXA_OPB_CASE(OP_JACOBI)
    HEXA_OPB_CASE(OP_CHEB2)
    default: break;
  }
#undef HEXA_OPB_CASE
}

template int op_batch_plan<double>(BatchInst*, int, int);
template int op_batch_plan<float>(BatchInst*, int, int);
template void launch_op_batch<double>(int, const BatchOpArgs<double>&, bool, cudaStream_t);
template void launch_op_batch<float>(int, const BatchOpArgs<float>&, bool, cudaStream_t);

template void launch_op<double>(int, const OpArgs<double>&, cudaStream_t);
template void launch_op<float>(int, const OpArgs<float>&, cudaStream_t);
template long long op_num_blocks<double>(const Grid&, int);
template long long op_num_blocks<float>(const Grid&, int);
template int op_pick_kchunk<double>(const Grid&);
template int op_pick_kchunk<float>(const Grid&);
template ModalK<float> cast_modal<float>(const ModalK<double>&);
template ModalK<double> cast_modal<double>(const ModalK<double>&);

ModalK<float> modal_to_f32(const ModalK<double>& K) { return cast_modal<float>(K); }

}  // namespace hexa
