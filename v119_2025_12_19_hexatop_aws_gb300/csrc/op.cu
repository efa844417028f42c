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
template <typename IX>
struct ColumnAddr {
  IX base;   // 3 * node index of corner 0 at layer 0
  IX row3;   // 3 * NX: corner 2 is one node row up
  IX plane3; // 3 * NX * NY
  bool ok[4];
};

template <typename IX>
__device__ __forceinline__ ColumnAddr<IX> column_addr(const Grid& g, int ie, int je) {
  ColumnAddr<IX> a;
  a.base = (IX)3 * ((IX)ie + (IX)g.NX * je);
  a.row3 = (IX)3 * g.NX;
  a.plane3 = (IX)3 * g.NX * g.NY;
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const int i = ie + (cc & 1), j = je + (cc >> 1);
    a.ok[cc] = (i >= 0) && (i < g.NX) && (j >= 0) && (j < g.NY);
  }
  return a;
}

// Corner values of the column at node layer kk; zeros outside the grid.
template <typename T, typename IX>
__device__ __forceinline__ void load_corners(const Grid& g, const ColumnAddr<IX>& ca, const T* __restrict__ x, int kk,
                                             T (&v)[4][3]) {
  const bool kok = (kk >= 0) && (kk < g.NZ);
  const IX lb = ca.base + ca.plane3 * (IX)kk;
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const bool ok = kok && ca.ok[cc];
    const IX o = lb + ((cc & 1) ? 3 : 0) + ((cc >> 1) ? ca.row3 : (IX)0);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[cc][c] = ok ? ldx(x + o + c) : T(0);
  }
}

// 1/d for the smoothers: correctly rounded in FP32; in FP64 a float seed and
// two Newton steps (relative error far below 1e-15, deterministic).
__device__ __forceinline__ float recip(float d) { return __frcp_rn(d); }
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

// CTA height in warps.  FP32: 16 warps, one CTA per SM (127 registers); 8-warp
// CTAs two per SM measured 5 % slower on the 384x192x192 Chebyshev step
// (359 us against 340 us), the larger halo outweighing the shorter barriers.
#ifndef HEXA_OP_TYW32
#define HEXA_OP_TYW32 16
#endif
#ifndef HEXA_OP_ASYNC
#define HEXA_OP_ASYNC 0
#endif
constexpr int kRingStages = 3, kRingSlots = 20;
template <typename T>
constexpr int op_tyw() { return sizeof(T) == 8 ? 8 : HEXA_OP_TYW32; }
#ifndef HEXA_OP_MINCTAS32
#define HEXA_OP_MINCTAS32 (HEXA_OP_TYW32 <= 8 ? 2 : 1)
#endif
template <typename T>
constexpr int op_min_ctas() { return sizeof(T) == 8 ? 1 : HEXA_OP_MINCTAS32; }
template <typename T, bool MULTI>
constexpr bool op_async() { return HEXA_OP_ASYNC && sizeof(T) == 4 && !MULTI; }

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

// FP32 operator loads staged through a per-thread shared-memory ring with
// cp.async (4-byte copies, zero-filled where masked), two node layers ahead:
// each thread copies exactly the 19 values it later reads (12 corner values,
// its element factor, b and the previous iterate at its node), so the ring
// needs no cross-thread synchronisation and the loads' latency is hidden
// without the registers a deeper register prefetch would take.

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// One work item: the node columns of tile (tx, ty) for node layers [k0, k1).
// IX is the index type: int whenever 3 * nNodes fits, which halves the
// integer work of the address arithmetic.
template <typename T, int MODE, int TYW, typename IX, typename A, bool ASYNC = false>
__device__ __forceinline__ void op_item(const A& a, int tx, int ty, int chunk,
                                        T (&xch)[2][TYW][32][4],
                                        double& acc0, long long co, float* ring = nullptr) {
  constexpr int NX_OWN = 31, NY_OWN = TYW - 1;
  constexpr bool NEED_F = (MODE == OP_JACOBI || MODE == OP_CHEB2);
  const Grid& g = a.g;
  const int lane = threadIdx.x, wy = threadIdx.y;
  const int i0 = tx * NX_OWN, j0 = ty * NY_OWN;
  const int k0 = chunk * a.kchunk;
  const int k1 = min(k0 + a.kchunk, g.NZ);
  const int ie = i0 - 1 + lane, je = j0 - 1 + wy;
  const bool colv = (ie >= 0) && (ie < g.nx) && (je >= 0) && (je < g.ny);
  const IX ecol = colv ? ((IX)ie + (IX)g.nx * je) : (IX)0;
  const IX eplane = (IX)g.nx * g.ny;
  const int in = i0 + lane, jn = j0 + wy;
  const bool own = (lane < NX_OWN) && (wy < NY_OWN) && (in < g.NX) && (jn < g.NY);
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
  const unsigned colfix = (((F & 1u) && in == 0) || ((F & 2u) && in == g.NX - 1) || ((F & 4u) && jn == 0) ||
                           ((F & 8u) && jn == g.NY - 1)) ? 7u : 0u;
  const IX nplane = (IX)g.NX * g.NY;
  const IX ncol = (IX)in + (IX)g.NX * jn;

  auto facload = [&](int k) -> T {
    return (colv && k >= 0 && k < g.nz) ? ldx(fac + ecol + eplane * k) : T(0);
  };
  // ---- staged loads (ASYNC): ring slot q of node layer kk for this thread
  constexpr int NT = 32 * TYW;
  const int tid = lane + 32 * wy;
  auto rslot = [&](int kk, int q) -> float* {
    const int st = ((kk % kRingStages) + kRingStages) % kRingStages;
    return ring + (st * kRingSlots + q) * NT + tid;
  };
  constexpr bool NEED_B = MODE == OP_RESID || MODE == OP_RESID_NORM || MODE == OP_JACOBI || MODE == OP_CHEB2;
  auto issue = [&](int kk) {  // node layer kk: corners, element factor kk, b and x_prev at the own node
    if constexpr (ASYNC) {
      const bool kok = (kk >= 0) && (kk < g.NZ);
      const IX lb = ca.base + ca.plane3 * (IX)kk;
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const bool ok = kok && ca.ok[cc];
        const IX o = ok ? lb + ((cc & 1) ? 3 : 0) + ((cc >> 1) ? ca.row3 : (IX)0) : (IX)0;
#pragma unroll
        for (int c = 0; c < 3; ++c) cp_async4(rslot(kk, 3 * cc + c), (const float*)x + o + c, ok);
      }
      const bool fok = colv && kk >= 0 && kk < g.nz;
      cp_async4(rslot(kk, 12), (const float*)fac + (fok ? ecol + eplane * kk : (IX)0), fok);
      if (NEED_B) {
        const bool bok = own && kok;
        const IX nb3 = bok ? (IX)3 * (ncol + nplane * (IX)kk) : (IX)0;
#pragma unroll
        for (int c = 0; c < 3; ++c) cp_async4(rslot(kk, 13 + c), (const float*)bv + nb3 + c, bok);
        if (MODE == OP_CHEB2) {
          const bool pok = bok && xinv;
#pragma unroll
          for (int c = 0; c < 3; ++c) cp_async4(rslot(kk, 16 + c), pok ? (const float*)xinv + nb3 + c : (const float*)x, pok);
        }
      }
      cp_async_commit();
    }
  };
  auto corners = [&](int kk, T (&v)[4][3]) {
    if constexpr (ASYNC) {
#pragma unroll
      for (int cc = 0; cc < 4; ++cc)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[cc][c] = *rslot(kk, 3 * cc + c);
    } else {
      load_corners<T, IX>(g, ca, x, kk, v);
    }
  };
  auto facval = [&](int kk) -> T {
    if constexpr (ASYNC) return *rslot(kk, 12);
    else return facload(kk);
  };

  T Lm[4][3], carry[4][3], xown[3];
  T fprev;
  if constexpr (ASYNC) {
    issue(k0 - 1);
    issue(k0);
    issue(k0 + 1);
    cp_async_wait1();  // layers k0-1 and k0 have landed
  }
  {
    T raw[4][3];
    corners(k0 - 1, raw);
    T Lprev[4][3];
    xy_forward<T>(raw, Lprev);
    corners(k0, raw);
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
    xy_forward<T>(raw, Lm);
    fprev = facval(k0 - 1);
    T lo[4][3];
    element_modal<T>(a.K, Lprev, Lm, fprev, lo, carry);
  }

  // sums of this item in the kernel's own precision (one item is at most a
  // few dozen layers per thread), folded into the FP64 accumulator at the end:
  // FP64 arithmetic in the FP32 kernels would run at GB300's FP64 rate
  T accT = T(0);
  T nraw[4][3];
  T fnext = T(0);
  if constexpr (!ASYNC) {
    load_corners<T, IX>(g, ca, x, k0 + 1, nraw);
    fnext = facload(k0);
  }

#pragma unroll 2
  for (int k = k0; k < k1; ++k) {
    T raw[4][3];
    T f;
    if constexpr (ASYNC) {
      if (k + 2 <= k1) issue(k + 2);  // into the slot layer k-1 used
      else cp_async_commit();          // empty group keeps the wait count uniform
      cp_async_wait1();                // layers k and k+1 have landed
      corners(k + 1, raw);
      f = facval(k);
    } else {
#pragma unroll
      for (int cc = 0; cc < 4; ++cc)
#pragma unroll
        for (int c = 0; c < 3; ++c) raw[cc][c] = nraw[cc][c];
      f = fnext;
      if (k + 1 < k1) {  // prefetch the next layer
        load_corners<T, IX>(g, ca, x, k + 2, nraw);
        fnext = facload(k + 1);
      }
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
    store4(&xch[buf][wy][lane][0], T0[0], T0[1], T0[2], F1);  // one vector store, no bank conflicts
    __syncthreads();
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
        if (MODE == OP_APPLY) {
          out = fixd ? T(0) : Ax;
        } else if (MODE == OP_APPLY_DOT) {
          out = fixd ? T(0) : Ax;
          accT = fma(xown[c], out, accT);
        } else if (MODE == OP_RESID || MODE == OP_RESID_NORM) {
          const T bvc = ASYNC ? (T)*rslot(k, 13 + c) : ldx(bv + 3 * n + c);
          out = fixd ? T(0) : (bvc - Ax);
          if (MODE == OP_RESID_NORM) accT = fma(out, out, accT);
        } else if (MODE == OP_JACOBI) {  // x + omega (b - Ax) / D
          const T bvc = ASYNC ? (T)*rslot(k, 13 + c) : ldx(bv + 3 * n + c);
          out = fixd ? T(0) : fma(a.omega * dinv[c], bvc - Ax, xown[c]);
        } else {  // OP_CHEB2: x + c1 (x - x_prev) + c2 D^-1 (b - Ax)
          // plain load: y may alias xin (the staged copy was taken before this thread's write)
          const T xp = ASYNC ? (T)*rslot(k, 16 + c) : (xinv ? xinv[3 * n + c] : T(0));
          const T bvc = ASYNC ? (T)*rslot(k, 13 + c) : ldx(bv + 3 * n + c);
          const T t = fma(a.c1, xown[c] - xp, xown[c]);
          out = fixd ? T(0) : fma(a.c2 * dinv[c], bvc - Ax, t);
        }
        yv[3 * n + c] = out;
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) xown[c] = raw[3][c];
  }

  acc0 += (double)accT;
  if constexpr (ASYNC) cp_async_wait0();
  __syncthreads();  // the next item reuses xch
}

template <typename T, int MODE, int TYW, typename IX, bool MULTI>
__global__ void __launch_bounds__(32 * TYW, op_min_ctas<T>()) op_kernel(const OpArgs<T> a) {
  if (a.halt && *((volatile const int*)a.halt)) return;
  __shared__ __align__(16) T xch[2][TYW][32][4];
  extern __shared__ __align__(16) float op_ring[];  // staged loads (FP32 single-column forms)
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
    } else {
      op_item<T, MODE, TYW, IX, OpArgs<T>, op_async<T, MULTI>()>(a, tx, ty, chunk, xch, acc0, 0, op_ring);
    }
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


// Dynamic shared memory of the staged-load ring (0 for the direct forms).
template <typename T, bool MULTI>
constexpr int op_ring_bytes() {
  return op_async<T, MULTI>() ? kRingStages * kRingSlots * 32 * op_tyw<T>() * (int)sizeof(float) : 0;
}

// Raises the kernel's dynamic shared-memory limit to the ring size, once.
template <typename T, int MODE, typename IX, bool MULTI>
static void op_prepare() {
  static bool done = false;
  if (!done) {
    if (op_ring_bytes<T, MULTI>() > 0)
      cudaFuncSetAttribute(op_kernel<T, MODE, op_tyw<T>(), IX, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           op_ring_bytes<T, MULTI>());
    done = true;
  }
}

template <typename T, int MODE>
static int op_resident_ctas() {
  static int cached = 0;
  if (!cached) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    op_prepare<T, MODE, long long, false>();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, op_kernel<T, MODE, op_tyw<T>(), long long, false>,
                                                  32 * op_tyw<T>(), op_ring_bytes<T, false>());
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

template <typename T>
void launch_op(int mode, const OpArgs<T>& a0, cudaStream_t st) {
  constexpr int TYW = op_tyw<T>();
  OpArgs<T> a = a0;
  op_tiles<T>(a.g, a.kchunk, &a.tiles_x, &a.tiles_y, &a.nchunks);
  const long long items = (long long)a.tiles_x * a.tiles_y * a.nchunks;
  const int grid = (int)std::min<long long>(items, resident_ctas<T>(mode));
  const dim3 block(32, TYW);
  const bool i32 = a.g.ndof() < (1LL << 30) && a.g.nelem() < (1LL << 30);
  if (a.ncol > 1) {  // multi-column forms: the plain apply and the residual
    if (mode == OP_APPLY) {
      if (i32) op_kernel<T, OP_APPLY, TYW, int, true><<<grid, block, 0, st>>>(a);
      else op_kernel<T, OP_APPLY, TYW, long long, true><<<grid, block, 0, st>>>(a);
    } else if (mode == OP_RESID) {
      if (i32) op_kernel<T, OP_RESID, TYW, int, true><<<grid, block, 0, st>>>(a);
      else op_kernel<T, OP_RESID, TYW, long long, true><<<grid, block, 0, st>>>(a);
    }
    return;
  }
#define HEXA_OP_CASE(M)                                                                      \
  case M:                                                                                   \
    if (i32) {                                                                              \
      op_prepare<T, M, int, false>();                                                       \
      op_kernel<T, M, TYW, int, false><<<grid, block, op_ring_bytes<T, false>(), st>>>(a);  \
    } else {                                                                                \
      op_prepare<T, M, long long, false>();                                                 \
      op_kernel<T, M, TYW, long long, false><<<grid, block, op_ring_bytes<T, false>(), st>>>(a); \
    }                                                                                       \
    break;
  switch (mode) {
    HEXA_OP_CASE(OP_APPLY)
    HEXA_OP_CASE(OP_APPLY_DOT)
    HEXA_OP_CASE(OP_RESID)
    HEXA_OP_CASE(OP_RESID_NORM)
    HEXA_OP_CASE(OP_JACOBI)
    HEXA_OP_CASE(OP_CHEB2)
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
void launch_op_batch(int mode, const BatchOpArgs<T>& a, bool idx32, cudaStream_t st) {
  constexpr int TYW = op_tyw<T>();
  const dim3 block(32, TYW);
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
