// Host orchestration of the solve path: workspace cache, the PCG driver with
// device-resident scalars (optionally replayed from CUDA graphs), the
// geometric-multigrid V-cycle, the reference's shift/fallback control flow
// and the mixed-precision refinement loop.
//
// Control flow restated from src/Solvers/GPUSolver.jl:182-465:
//   - sigma = shift_factor * max(diag K_ff)                        (:343)
//   - up to max_shift_attempts attempts, shift *= shift_multiplier  (:342-432)
//   - first attempt starts from u_guess, later ones from zero       (:347-351)
//   - NaN or divergence (rel > 10, or k > 500 and rel > 100 best) under
//     multigrid restarts with Jacobi                                (:387-401,434-437)
//   - stagnation acceptance of the best iterate when best < stagnation_tol
//                                                                   (:426-430)
//   - otherwise the best iterate is returned as not converged       (:439-443)
// New here: the FP64 true residual ||f-(K+sI)u||/||f|| is recomputed after
// convergence and the iteration continues until it meets the tolerance.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <vector>

#include "element.h"
#include "hexa_kernels.h"
#include "solver.h"

namespace hexa {

void launch_scalars_init(PcgScalars* s, const PcgScalars* parent, int max_iter, cudaStream_t st, int ncol = 1);

// ------------------------------------------------------------------ context
void* Ctx::get(const std::string& name, size_t bytes) {
  if (bytes == 0) bytes = 16;
  auto it = bufs.find(name);
  if (it != bufs.end() && it->second.second >= bytes) return it->second.first;
  if (it != bufs.end()) {
    cudaFreeAsync(it->second.first, st);
    bufs.erase(it);
  }
  void* p = nullptr;
  if (cudaMallocAsync(&p, bytes, st) != cudaSuccess) {
    cudaGetLastError();
    err = "device allocation of " + std::to_string(bytes) + " bytes failed (" + name + ")";
    return nullptr;
  }
  bufs[name] = {p, bytes};
  return p;
}

bool Ctx::ensure_partials(size_t n) {
  if (n <= partials_cap) return true;
  void* p = get("partials", n * sizeof(double));
  if (!p) return false;
  partials = (double*)p;
  partials_cap = n;
  return true;
}

bool Ctx::cuda_ok(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return true;
  err = std::string(where) + ": " + cudaGetErrorString(e);
  return false;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool build_modal(double dx, double dy, double dz, double nu, ModalK<double>* K, std::string* err) {
  double ke[576];
  if (canonical_stiffness(dx, dy, dz, nu, ke) != 0) {
    if (err) *err = "invalid element geometry or Poisson ratio";
    return false;
  }
  double dropped = 0.0;
  if (modal_blocks(ke, K, &dropped) != 0) {
    if (err) *err = "K0 is not block diagonal in the Hadamard basis";
    return false;
  }
  return true;
}

// --------------------------------------------------------------- utilities
namespace {

constexpr int kRedBlocks = 152 * 4;  // grid of reducing vector passes
// Coarsest grids up to this many elements are solved by the single-CTA kernel.
constexpr long long kCoarseOneCta = 4096;

template <typename T>
struct Is64 { static constexpr bool v = sizeof(T) == 8; };

template <typename T>
int pick_kchunk(const Grid& g) {
  return op_pick_kchunk<T>(g);
}

RedArgs red(Ctx& c, int op, int nsum, PcgScalars* s, double* dst = nullptr) {
  RedArgs r;
  r.partials = c.partials;
  r.ticket = c.ticket;
  r.dst = dst;
  r.s = s;
  r.op = op;
  r.nsum = nsum;
  return r;
}

template <typename T>
struct Lev {
  Grid g;
  Mask m;
  T* fac = nullptr;
  T* xa = nullptr;  // level solution (coarse levels)
  T* xb = nullptr;  // smoother ping-pong
  T* b = nullptr;   // level right-hand side (coarse levels)
  T* r = nullptr;   // level residual
  T* dinv = nullptr, *p = nullptr, *q = nullptr, *z = nullptr;  // coarsest-level PCG
  T* w = nullptr;  // element-product scratch of the single-CTA coarse solve
  T* ainv = nullptr;  // dense inverse of the coarsest operator (small coarse grids)
  T* xw = nullptr, *bw = nullptr;  // W-cycle: second correction and its right-hand side
  T sigma = 0;
  int kchunk = 4;
};

template <typename T>
struct MG {
  std::vector<Lev<T>> L;
  ModalK<T> K;
  int quirk = 0;
  T omega = T(0.6);
  int nu1 = 2, nu2 = 2, citers = 30;
  int gamma = 1;  // coarse-grid visits per level (1: V-cycle, 2: W-cycle)
  int smoother = HEXA_SMOOTH_CHEBYSHEV;
  // Chebyshev on [lmax/ratio, lmax] of D^-1 A (ratio 10 by default): d_0 = D^-1 r / theta,
  // d_s = c1[s] d_{s-1} + c2[s] D^-1 r_s
  T inv_theta = T(0);
  std::vector<T> c1, c2;
  std::vector<double> ke;  // FP64 K0 of the fine element (dense coarse inverse)

  void set_chebyshev(double lmax, int nmax, double ratio) {
    const double lmin = lmax / ratio, th = 0.5 * (lmax + lmin), de = 0.5 * (lmax - lmin), sg = th / de;
    double rho = 1.0 / sg;
    inv_theta = (T)(1.0 / th);
    c1.assign(nmax + 1, T(0));
    c2.assign(nmax + 1, T(0));
    for (int s = 1; s <= nmax; ++s) {
      const double rn = 1.0 / (2.0 * sg - rho);
      c1[s] = (T)(rn * rho);
      c2[s] = (T)(2.0 * rn / de);
      rho = rn;
    }
  }
};

template <typename T>
OpArgs<T> opargs(const Lev<T>& L, const ModalK<T>& K, int quirk, const T* x, const T* b, T* y, T omega,
                 const int* halt, RedArgs r) {
  OpArgs<T> a;
  a.g = L.g;
  a.m = L.m;
  a.x = x;
  a.fac = L.fac;
  a.b = b;
  a.y = y;
  a.K = K;
  a.sigma = L.sigma;
  a.omega = omega;
  a.kchunk = L.kchunk;
  a.diag_quirk = quirk;
  a.red = r;
  a.halt = halt;
  a.xin = nullptr;
  a.c1 = T(0);
  a.c2 = T(0);
  return a;
}

template <typename T>
void op(Ctx& c, int mode, const OpArgs<T>& a) {
  launch_op<T>(mode, a, c.st);
  c.launches++;
}

// Number of levels: requested, or automatic (halve while every axis is even
// and the coarse grid keeps at least 2 elements per axis, down to ~2k nodes).
int plan_levels(const Grid& g, int requested) {
  int nx = g.nx, ny = g.ny, nz = g.nz, lv = 1;
  const int maxlv = requested > 0 ? requested : 16;
  while (lv < maxlv) {
    if ((nx & 1) || (ny & 1) || (nz & 1) || nx < 4 || ny < 4 || nz < 4) break;
    if (requested <= 0 && (long long)(nx + 1) * (ny + 1) * (nz + 1) <= 2500) break;
    nx >>= 1; ny >>= 1; nz >>= 1;
    ++lv;
  }
  return lv;
}

template <typename T>
bool build_mg(Ctx& c, MG<T>& mg, const Grid& g0, const Mask& m0, const T* fac0, int nlev, const std::string& tag) {
  mg.L.clear();
  Lev<T> L0;
  L0.g = g0;
  L0.m = m0;
  L0.fac = const_cast<T*>(fac0);
  L0.kchunk = pick_kchunk<T>(g0);
  const long long n0 = g0.ndof();
  L0.xb = c.vec<T>(tag + "xb0", n0);
  L0.r = c.vec<T>(tag + "r0", n0);
  if (!L0.xb || !L0.r) return false;

  mg.L.push_back(L0);
  for (int l = 1; l < nlev; ++l) {
    const Lev<T>& F = mg.L[l - 1];
    Lev<T> C;
    C.g = make_grid(F.g.nx / 2, F.g.ny / 2, F.g.nz / 2);
    C.m.faces = F.m.faces;
    C.m.node = nullptr;
    const std::string s = tag + std::to_string(l);
    if (F.m.node) {
      uint8_t* mk = c.vec<uint8_t>(s + "mask", C.g.nnode());
      if (!mk) return false;
      launch_coarsen_mask(F.g, F.m.node, C.g, mk, c.st);
      c.launches++;
      C.m.node = mk;
    }
    C.fac = c.vec<T>(s + "fac", C.g.nelem());
    const long long n = C.g.ndof();
    C.xa = c.vec<T>(s + "xa", n);
    C.xb = c.vec<T>(s + "xb", n);
    C.b = c.vec<T>(s + "b", n);
    C.r = c.vec<T>(s + "r", n);
    if (!C.fac || !C.xa || !C.xb || !C.b || !C.r) return false;
    if (mg.gamma > 1) {
      C.xw = c.vec<T>(s + "xw", n);
      C.bw = c.vec<T>(s + "bw", n);
      if (!C.xw || !C.bw) return false;
    }
    launch_coarsen_factors<T>(F.g, F.fac, C.g, C.fac, c.st);
    c.launches++;
    C.kchunk = pick_kchunk<T>(C.g);
    mg.L.push_back(C);
  }
  Lev<T>& Lc = mg.L.back();
  const long long nc = Lc.g.ndof();
  const std::string s = tag + "c";
  Lc.dinv = c.vec<T>(s + "dinv", nc);
  Lc.p = c.vec<T>(s + "p", nc);
  Lc.q = c.vec<T>(s + "q", nc);
  Lc.z = c.vec<T>(s + "z", nc);
  if (Lc.g.nelem() <= kCoarseOneCta) {
    Lc.w = c.vec<T>(s + "w", 24 * Lc.g.nelem());
    if (!Lc.w) return false;
  }
  if (!Lc.xa) {  // single-level hierarchy
    Lc.xa = c.vec<T>(s + "xa", nc);
    Lc.b = c.vec<T>(s + "b", nc);
  }
  return Lc.dinv && Lc.p && Lc.q && Lc.z && Lc.xa;
}

// Coarsest grids of at most this many free DOFs are solved exactly by one
// dense matvec with the inverse of (K + sigma I) on their free DOFs (Cholesky
// and inverse in FP64 on the host at setup, about n^3 flops, well under 0.1 s
// at the limit); larger ones by the coarse PCG.  The count is of free DOFs:
// the 8x4x4 coarsest grid of a 256x128x128 hierarchy has 675 DOFs, 600 of
// them free once its x = 0 face is clamped.
constexpr long long kDenseCoarse = 640;

template <typename T>
void coarse_dense_setup(Ctx& c, MG<T>& mg, double sigma_c) {
  Lev<T>& V = mg.L.back();
  V.ainv = nullptr;
  const long long n = V.g.ndof();
  if (n > 4 * kDenseCoarse || mg.ke.size() != 576) return;
  const Grid& g = V.g;
  std::vector<T> fac(g.nelem());
  std::vector<uint8_t> mask;
  cudaMemcpyAsync(fac.data(), V.fac, sizeof(T) * fac.size(), cudaMemcpyDeviceToHost, c.st);
  if (V.m.node) {
    mask.resize(g.nnode());
    cudaMemcpyAsync(mask.data(), V.m.node, mask.size(), cudaMemcpyDeviceToHost, c.st);
  }
  if (cudaStreamSynchronize(c.st) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  // free DOFs: the device's fixed_bits (clamped faces, then the node mask)
  const uint32_t F = V.m.faces;
  std::vector<int> fidx(n, -1);
  int nf = 0;
  for (int k = 0; k < g.NZ; ++k)
    for (int j = 0; j < g.NY; ++j)
      for (int i = 0; i < g.NX; ++i) {
        const long long nd = i + (long long)g.NX * (j + (long long)g.NY * k);
        unsigned fx = (((F & 1u) && i == 0) || ((F & 2u) && i == g.NX - 1) || ((F & 4u) && j == 0) ||
                       ((F & 8u) && j == g.NY - 1) || ((F & 16u) && k == 0) || ((F & 32u) && k == g.NZ - 1))
                          ? 7u : 0u;
        if (!mask.empty()) fx |= mask[nd];
        for (int cc = 0; cc < 3; ++cc)
          if (!((fx >> cc) & 1u)) fidx[3 * nd + cc] = nf++;
      }
  if (nf == 0 || nf > kDenseCoarse) return;
  std::vector<double> A((size_t)nf * nf, 0.0);
  for (int q = 0; q < nf; ++q) A[(size_t)q * nf + q] = sigma_c;
  static const int ref_to_corner[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // K0 node order (Mesh.jl:45-53) -> dx + 2dy + 4dz
  long long dof[24];
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i) {
        const double f = (double)fac[i + (long long)g.nx * (j + (long long)g.ny * k)];
        for (int a = 0; a < 8; ++a) {
          const int cc = ref_to_corner[a];
          const long long nd = (i + (cc & 1)) + (long long)g.NX * ((j + ((cc >> 1) & 1)) + (long long)g.NY * (k + (cc >> 2)));
          for (int d = 0; d < 3; ++d) dof[3 * a + d] = fidx[3 * nd + d];
        }
        for (int r = 0; r < 24; ++r) {
          if (dof[r] < 0) continue;
          for (int q = 0; q < 24; ++q)
            if (dof[q] >= 0) A[(size_t)dof[r] * nf + dof[q]] += f * mg.ke[r + 24 * q];
        }
      }
  // Cholesky A = L L^T (lower, in place); give up (coarse PCG) on a non-positive pivot
  for (int jj = 0; jj < nf; ++jj) {
    double d = A[(size_t)jj * nf + jj];
    for (int m = 0; m < jj; ++m) d -= A[(size_t)jj * nf + m] * A[(size_t)jj * nf + m];
    if (!(d > 0.0)) return;
    const double ljj = std::sqrt(d);
    A[(size_t)jj * nf + jj] = ljj;
    for (int ii = jj + 1; ii < nf; ++ii) {
      double v = A[(size_t)ii * nf + jj];
      for (int m = 0; m < jj; ++m) v -= A[(size_t)ii * nf + m] * A[(size_t)jj * nf + m];
      A[(size_t)ii * nf + jj] = v / ljj;
    }
  }
  // inverse, column by column: L y = e_q, L^T x = y
  std::vector<double> inv((size_t)nf * nf), y(nf);
  for (int q = 0; q < nf; ++q) {
    for (int ii = 0; ii < nf; ++ii) {
      double v = ii == q ? 1.0 : 0.0;
      for (int m = q; m < ii; ++m) v -= A[(size_t)ii * nf + m] * y[m];
      y[ii] = ii < q ? 0.0 : v / A[(size_t)ii * nf + ii];
    }
    for (int ii = nf - 1; ii >= 0; --ii) {
      double v = y[ii];
      for (int m = ii + 1; m < nf; ++m) v -= A[(size_t)m * nf + ii] * y[m];
      y[ii] = v / A[(size_t)ii * nf + ii];
    }
    for (int ii = 0; ii < nf; ++ii) inv[(size_t)ii * nf + q] = y[ii];
  }
  // embed (zero rows/columns at fixed DOFs); symmetric, so either order reads coalesced
  std::vector<T> full((size_t)n * n, T(0));
  for (long long a = 0; a < n; ++a) {
    if (fidx[a] < 0) continue;
    for (long long b = 0; b < n; ++b)
      if (fidx[b] >= 0) full[(size_t)a * n + b] = (T)inv[(size_t)fidx[a] * nf + fidx[b]];
  }
  T* d = c.vec<T>(std::string(sizeof(T) == 8 ? "mgdense64" : "mgdense32"), (size_t)n * n);
  if (!d) {
    c.err.clear();
    return;
  }
  cudaMemcpyAsync(d, full.data(), sizeof(T) * full.size(), cudaMemcpyHostToDevice, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  V.ainv = d;
}

template <typename T>
void mg_set_shift(Ctx& c, MG<T>& mg, double sigma) {
  double s = sigma;
  for (size_t l = 0; l < mg.L.size(); ++l) {
    mg.L[l].sigma = (T)s;
    s *= 8.0;  // row sums of P^T P
  }
  Lev<T>& Lc = mg.L.back();
  launch_diag<T>(Lc.g, Lc.m, Lc.fac, mg.K, mg.quirk, Lc.sigma, nullptr, Lc.dinv, c.st);
  c.launches++;
  coarse_dense_setup<T>(c, mg, sigma * std::pow(8.0, (double)(mg.L.size() - 1)));
}

template <typename T>
void coarse_solve(Ctx& c, MG<T>& mg, const T* b, T* x, const int* halt_main) {
  Lev<T>& V = mg.L.back();
  const long long n = V.g.ndof();
  if (V.ainv) {  // exact: one dense matvec
    launch_dense_coarse<T>(n, V.ainv, b, x, halt_main, c.st);
    c.launches++;
    return;
  }
  if (V.w) {
    launch_coarse_pcg<T>(V.g, V.m, V.fac, mg.K, V.sigma, V.dinv, b, x, V.r, V.z, V.p, V.q, V.w, mg.citers, halt_main,
                         c.st);
    c.launches++;
    return;
  }
  launch_scalars_init(c.s2, c.s, mg.citers, c.st);
  launch_fill<T>(x, T(0), n, c.st);
  launch_copy<T>(V.r, b, n, c.st);
  c.launches += 3;
  launch_jacobi_precond<T>(V.z, V.r, V.dinv, n, red(c, FIN_INIT_RZ, 1, c.s2), kRedBlocks, &c.s2->halt, c.st);
  launch_copy<T>(V.p, V.z, n, c.st);
  c.launches += 2;
  const int* h2 = &c.s2->halt;
  for (int it = 0; it < mg.citers; ++it) {
    op<T>(c, OP_APPLY_DOT, opargs<T>(V, mg.K, mg.quirk, V.p, nullptr, V.q, T(0), h2, red(c, FIN_PCG_ALPHA, 1, c.s2)));
    launch_pcg_update<T>(x, V.r, V.z, V.p, V.q, V.dinv, n, red(c, FIN_PCG_RES, 2, c.s2), kRedBlocks, c.s2, c.st);
    launch_p_update<T>(V.p, V.z, n, c.s2, c.st);
    c.launches += 2;
  }
  (void)halt_main;
}

// One V-cycle from level l.  With fin given, the last post-smoothing step
// of the cycle also sums b.x_out (r.z of the flexible PCG) into that reduction;
// returns whether it did.
template <typename T>
bool vcycle(Ctx& c, MG<T>& mg, int l, const T* b, T* xout, const int* halt, const RedArgs* fin = nullptr) {
  Lev<T>& V = mg.L[l];
  if (l == (int)mg.L.size() - 1) {
    coarse_solve<T>(c, mg, b, xout, halt);
    return false;
  }
  // x buffers alternate between xout and V.xb so that the last write lands in xout
  const int nw = mg.nu1 + mg.nu2;
  auto bufw = [&](int w) -> T* { return ((nw - 1 - w) % 2 == 0) ? xout : V.xb; };
  int w = 0;
  T* cur = bufw(w++);
  RedArgs none = red(c, FIN_NONE, 1, nullptr);
  const bool cheb = mg.smoother == HEXA_SMOOTH_CHEBYSHEV;
  // Chebyshev step s >= 1: x_{s+1} = x_s + c1 (x_s - x_{s-1}) + c2 D^-1 (b - A x_s),
  // written over x_{s-1} (the buffer bufw() hands out next)
  const T* prev = nullptr;
  auto cheb_step = [&](int s) {
    T* nx = bufw(w++);
    OpArgs<T> a = opargs<T>(V, mg.K, mg.quirk, cur, b, nx, T(0), halt, none);
    a.xin = prev;
    a.c1 = mg.c1[s];
    a.c2 = mg.c2[s];
    op<T>(c, OP_CHEB2, a);
    prev = cur;
    cur = nx;
  };
  // the first sweep from zero is D^-1 b scaled by omega (damped Jacobi) or 1/theta (Chebyshev)
  launch_jacobi0<T>(V.g, V.m, V.fac, mg.K, mg.quirk, V.sigma, cheb ? mg.inv_theta : mg.omega, b, cur, halt, c.st);
  c.launches++;
  for (int s = 1; s < mg.nu1; ++s) {
    if (cheb) {
      cheb_step(s);
    } else {
      T* nx = bufw(w++);
      op<T>(c, OP_JACOBI, opargs<T>(V, mg.K, mg.quirk, cur, b, nx, mg.omega, halt, none));
      cur = nx;
    }
  }
  op<T>(c, OP_RESID, opargs<T>(V, mg.K, mg.quirk, cur, b, V.r, mg.omega, halt, none));
  Lev<T>& C = mg.L[l + 1];
  launch_restrict<T>(V.g, V.r, C.g, C.m, C.b, halt, c.st);
  c.launches++;
  vcycle<T>(c, mg, l + 1, C.b, C.xa, halt);
  if (mg.gamma > 1 && C.xw && l + 2 < (int)mg.L.size()) {
    // W-cycle: a second cycle on the coarse residual (its own right-hand side
    // and output buffers: the cycle reuses the level's r and xb), added to the
    // first correction
    op<T>(c, OP_RESID, opargs<T>(C, mg.K, mg.quirk, C.xa, C.b, C.bw, T(0), halt, none));
    vcycle<T>(c, mg, l + 1, C.bw, C.xw, halt);
    launch_axpby<T>(C.xa, T(1), C.xw, T(1), C.g.ndof(), c.st);
    c.launches++;
  }
  launch_prolong_add<T>(C.g, C.xa, V.g, V.m, cur, halt, c.st);
  c.launches++;
  bool fused = false;
  for (int s = 0; s < mg.nu2; ++s) {
    const bool last = fin && s == mg.nu2 - 1;
    if (cheb && s > 0) {
      if (last) {
        T* nx = bufw(w++);
        OpArgs<T> a = opargs<T>(V, mg.K, mg.quirk, cur, b, nx, T(0), halt, *fin);
        a.xin = prev;
        a.c1 = mg.c1[s];
        a.c2 = mg.c2[s];
        op<T>(c, OP_CHEB2_DOT, a);
        prev = cur;
        cur = nx;
      } else {
        cheb_step(s);
      }
    } else {  // damped Jacobi, or the first Chebyshev step (omega = 1/theta)
      T* nx = bufw(w++);
      op<T>(c, last ? OP_JACOBI_DOT : OP_JACOBI,
            opargs<T>(V, mg.K, mg.quirk, cur, b, nx, cheb ? mg.inv_theta : mg.omega, halt, last ? *fin : none));
      prev = cur;
      cur = nx;
    }
    fused = fused || last;
  }
  return fused;
}

// A CUDA graph replaying a fixed launch sequence.
struct Graph {
  cudaGraphExec_t exec = nullptr;
  int64_t nodes = 0;
  ~Graph() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    nodes = 0;
  }
};

// k columns through one V-cycle together (the block PCG's preconditioner):
// the smoothing and residual launches of a level run over all k columns (each
// work item applies the columns in turn while its element factors sit in
// L1, one launch instead of k); the first sweep, the transfers and the
// coarsest-level solve run per column.  Column j of every buffer starts at
// j * (the level's DOF count).  The same arithmetic as k calls of vcycle
// without a fused reduction.
template <typename T>
struct ColBufs {
  std::vector<T*> xa, xb, b, r;  // per level, k columns each
};

template <typename T>
void vcycle_cols(Ctx& c, MG<T>& mg, ColBufs<T>& cb, int l, const T* b, T* xout, int k, const int* halt) {
  Lev<T>& V = mg.L[l];
  const long long n = V.g.ndof();
  if (l == (int)mg.L.size() - 1) {
    if (V.ainv) {  // exact: one dense multiply for all k columns
      launch_dense_coarse<T>(n, V.ainv, b, xout, halt, c.st, k);
      c.launches++;
      return;
    }
    for (int j = 0; j < k; ++j) coarse_solve<T>(c, mg, b + j * n, xout + j * n, halt);
    return;
  }
  const int nw = mg.nu1 + mg.nu2;
  T* xbk = cb.xb[l];
  auto bufw = [&](int w) -> T* { return ((nw - 1 - w) % 2 == 0) ? xout : xbk; };
  int w = 0;
  T* cur = bufw(w++);
  const RedArgs none = red(c, FIN_NONE, 1, nullptr);
  const bool cheb = mg.smoother == HEXA_SMOOTH_CHEBYSHEV;
  const T* prev = nullptr;
  auto opk = [&](int mode, const T* x, T* y, const T* xin, T c1, T c2, T omega) {
    OpArgs<T> a = opargs<T>(V, mg.K, mg.quirk, x, b, y, omega, halt, none);
    a.xin = xin;
    a.c1 = c1;
    a.c2 = c2;
    a.ncol = k;
    op<T>(c, mode, a);
  };
  c.launches +=
      launch_jacobi0<T>(V.g, V.m, V.fac, mg.K, mg.quirk, V.sigma, cheb ? mg.inv_theta : mg.omega, b, cur, halt, c.st, k);
  for (int s = 1; s < mg.nu1; ++s) {
    T* nx = bufw(w++);
    if (cheb) {
      opk(OP_CHEB2, cur, nx, prev, mg.c1[s], mg.c2[s], T(0));
      prev = cur;
    } else {
      opk(OP_JACOBI, cur, nx, nullptr, T(0), T(0), mg.omega);
    }
    cur = nx;
  }
  opk(OP_RESID, cur, cb.r[l], nullptr, T(0), T(0), mg.omega);
  Lev<T>& C = mg.L[l + 1];
  c.launches += launch_restrict<T>(V.g, cb.r[l], C.g, C.m, cb.b[l + 1], halt, c.st, k);
  vcycle_cols<T>(c, mg, cb, l + 1, cb.b[l + 1], cb.xa[l + 1], k, halt);
  c.launches += launch_prolong_add<T>(C.g, cb.xa[l + 1], V.g, V.m, cur, halt, c.st, k);
  for (int s = 0; s < mg.nu2; ++s) {
    T* nx = bufw(w++);
    if (cheb && s > 0) {
      opk(OP_CHEB2, cur, nx, prev, mg.c1[s], mg.c2[s], T(0));
    } else {  // damped Jacobi, or the first Chebyshev step (omega = 1/theta)
      opk(OP_JACOBI, cur, nx, nullptr, T(0), T(0), cheb ? mg.inv_theta : mg.omega);
    }
    prev = cur;
    cur = nx;
  }
}

template <class F>
bool capture(Ctx& c, Graph& G, F&& body) {
  G.reset();
  if (cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return c.cuda_ok("capture begin");
  const int64_t before = c.launches;
  body();
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(c.st, &graph);
  G.nodes = c.launches - before;
  c.launches = before;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return c.fail(std::string("graph capture failed: ") + cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&G.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    G.exec = nullptr;
    return c.fail(std::string("graph instantiate failed: ") + cudaGetErrorString(e));
  }
  return true;
}

bool replay(Ctx& c, Graph& G) {
  if (cudaGraphLaunch(G.exec, c.st) != cudaSuccess) return c.cuda_ok("graph launch");
  c.launches += G.nodes;
  return true;
}

// PCG on (K + sigma I) x = b over one level-0 grid in precision T.
template <typename T>
struct PcgEnv {
  Lev<T>* L0 = nullptr;
  MG<T>* mg = nullptr;  // null: Jacobi
  ModalK<T> K;
  int quirk = 0;
  long long n = 0;
  T *x = nullptr, *r = nullptr, *zA = nullptr, *zB = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
  const T* b = nullptr;
  T* bestx = nullptr;  // nullable
  bool use_graphs = true;
  int graph_iters = 10;
};

struct PcgOut {
  int status = 0;  // PcgScalars::status
  int iters = 0;
  double relres = 0.0;
  double best_rel = INFINITY;
  double fine_applies = 0.0;
};

template <typename T>
void pcg_iteration(Ctx& c, PcgEnv<T>& E, int parity) {
  Lev<T>& L = *E.L0;
  const int* halt = &c.s->halt;
  op<T>(c, OP_APPLY_DOT, opargs<T>(L, E.K, E.quirk, E.p, nullptr, E.q, T(0), halt, red(c, FIN_PCG_ALPHA, 1, c.s)));
  if (!E.mg) {
    launch_pcg_update<T>(E.x, E.r, E.zA, E.p, E.q, E.dinv, E.n, red(c, FIN_PCG_RES, 2, c.s), kRedBlocks, c.s, c.st);
    launch_p_update<T>(E.p, E.zA, E.n, c.s, c.st);
    c.launches += 2;
  } else {
    T* zc = (parity == 0) ? E.zB : E.zA;
    T* zo = (parity == 0) ? E.zA : E.zB;
    // flexible beta = (r.z_new - r.z_old) / rz: r.z_old comes with the update
    // pass, r.z_new with the V-cycle's last smoothing step (no separate dot pass)
    launch_pcg_update_mg<T>(E.x, E.r, E.p, E.q, zo, E.n, red(c, FIN_PCG_RES_MG, 2, c.s), kRedBlocks, c.s, c.st);
    c.launches++;
    const RedArgs fin = red(c, FIN_PCG_BETA_RZ, 1, c.s);
    if (!vcycle<T>(c, *E.mg, 0, E.r, zc, halt, &fin)) {
      launch_dot<T>(E.r, zc, E.r, zo, E.n, red(c, FIN_PCG_BETA, 2, c.s), kRedBlocks, halt, c.st);
      c.launches++;
    }
    launch_p_update<T>(E.p, zc, E.n, c.s, c.st);
    c.launches++;
  }
}

template <typename T>
double applies_per_iteration(const PcgEnv<T>& E) {
  if (!E.mg) return 1.0;
  // fine-level operator passes: PCG apply + (nu1-1) + residual + nu2 ; the
  // coarser levels add ~1/8 per level
  const MG<T>& mg = *E.mg;
  double per = 0.0, w = 1.0;
  for (size_t l = 0; l + 1 < mg.L.size(); ++l) {
    per += w * (mg.nu1 - 1 + 1 + mg.nu2);
    w /= 8.0;
  }
  per += w * mg.citers;
  return 1.0 + per;
}

template <typename T>
double applies_per_iteration_mg(const MG<T>* mg) {
  PcgEnv<T> E;
  E.mg = const_cast<MG<T>*>(mg);
  return applies_per_iteration(E);
}

// Replays groups of PCG iterations (a CUDA graph captured on first use, or
// direct launches) until the device-side halt flag is set; *h receives the
// final scalars.  Iterations continue from whatever state E and c.s hold.
template <typename T>
bool pcg_drive(Ctx& c, PcgEnv<T>& E, Graph& graph, PcgScalars* h, double* ms = nullptr) {
  int G = E.graph_iters < 2 ? 2 : E.graph_iters;
  if (G & 1) ++G;  // even: each group starts with the same z / z_old buffer parity
  if (E.use_graphs && !graph.exec) {
    if (!capture(c, graph, [&]() {
          for (int i = 0; i < G; ++i) pcg_iteration<T>(c, E, i & 1);
        }))
      return false;
  }
  double host_best = INFINITY;
  if (ms) cudaEventRecord(c.ev[2], c.st);
  while (true) {
    if (E.use_graphs) {
      if (!replay(c, graph)) return false;
    } else {
      for (int i = 0; i < G; ++i) pcg_iteration<T>(c, E, i & 1);
      if (!c.cuda_ok("pcg iteration")) return false;
    }
    cudaMemcpyAsync(c.hs, c.s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess) return c.cuda_ok("pcg sync");
    *h = *c.hs;
    if (E.bestx && h->best_rel < host_best) {
      host_best = h->best_rel;
      cudaMemcpyAsync(E.bestx, E.x, sizeof(T) * E.n, cudaMemcpyDeviceToDevice, c.st);
    }
    if (h->halt) break;
  }
  if (ms) {
    cudaEventRecord(c.ev[3], c.st);
    cudaEventSynchronize(c.ev[3]);
    float t = 0.f;
    cudaEventElapsedTime(&t, c.ev[2], c.ev[3]);
    *ms += t;
  }
  return true;
}

// Runs PCG from the current E.x.  host_scalars carries tol/max_iter/cadence.
template <typename T>
bool run_pcg(Ctx& c, PcgEnv<T>& E, double tol, int max_iter, int cadence, bool x_is_zero, double bnorm,
             bool div_check, PcgOut* out, double* ms = nullptr) {
  PcgScalars h;
  std::memset(&h, 0, sizeof(h));
  h.tol = tol;
  h.max_iter = max_iter;
  h.cadence = cadence;
  h.bnorm = bnorm;
  h.best_rel = INFINITY;
  h.no_div = div_check ? 0 : 1;
  *c.hs = h;
  cudaMemcpyAsync(c.s, c.hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, c.st);
  Lev<T>& L = *E.L0;
  const int* halt = &c.s->halt;
  if (x_is_zero) {
    launch_copy<T>(E.r, E.b, E.n, c.st);
    c.launches++;
  } else {
    op<T>(c, OP_RESID_NORM, opargs<T>(L, E.K, E.quirk, E.x, E.b, E.r, T(0), halt, red(c, FIN_INIT_RES, 1, c.s)));
  }
  if (!E.mg) {
    launch_jacobi_precond<T>(E.zA, E.r, E.dinv, E.n, red(c, FIN_INIT_RZ, 1, c.s), kRedBlocks, halt, c.st);
    c.launches++;
  } else {
    vcycle<T>(c, *E.mg, 0, E.r, E.zA, halt);
    launch_dot<T>(E.r, E.zA, (const T*)nullptr, (const T*)nullptr, E.n, red(c, FIN_INIT_RZ, 1, c.s), kRedBlocks,
                  halt, c.st);
    c.launches++;
  }
  launch_copy<T>(E.p, E.zA, E.n, c.st);
  c.launches++;
  if (!c.cuda_ok("pcg setup")) return false;

  Graph graph;
  const int iter0 = 0;
  if (!pcg_drive<T>(c, E, graph, &h, ms)) return false;
  out->status = h.status;
  out->iters = h.iter - iter0;
  out->relres = h.relres;
  out->best_rel = h.best_rel;
  out->fine_applies += applies_per_iteration(E) * out->iters + (x_is_zero ? 0.0 : 1.0);
  return true;
}

template <typename T>
struct Host {
  static const T* fac(Ctx& c, const Problem& P) {
    T* f = c.vec<T>("fac_T", P.g.nelem());
    if (f) {
      launch_convert<T, double>(f, P.fac64, P.g.nelem(), c.st);
      c.launches++;
    }
    return f;
  }
};
template <>
struct Host<double> {
  static const double* fac(Ctx&, const Problem& P) { return P.fac64; }
};

// sqrt(||f - (K+sigma I) u||^2) in FP64, written to r64 as well.
double true_residual_norm(Ctx& c, const Problem& P, const ModalK<double>& K64, int quirk, double sigma, const double* u,
                          double* r64) {
  Lev<double> L;
  L.g = P.g;
  L.m = P.m;
  L.fac = const_cast<double*>(P.fac64);
  L.sigma = sigma;
  L.kchunk = pick_kchunk<double>(P.g);
  op<double>(c, OP_RESID_NORM, opargs<double>(L, K64, quirk, u, P.f64, r64, 0.0, nullptr, red(c, FIN_STORE, 1, nullptr, c.dscal + 8)));
  cudaMemcpyAsync(c.hscal + 8, c.dscal + 8, sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return std::sqrt(std::fmax(c.hscal[8], 0.0));
}

double device_dot(Ctx& c, const double* a, const double* b, long long n, int slot) {
  launch_dot<double>(a, b, (const double*)nullptr, (const double*)nullptr, n, red(c, FIN_STORE, 1, nullptr, c.dscal + slot),
                     kRedBlocks, nullptr, c.st);
  c.launches++;
  cudaMemcpyAsync(c.hscal + slot, c.dscal + slot, sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  return c.hscal[slot];
}

// Element bound on lambda_max(D^-1 A) for the smoothers (see smoother_bound).
double smoother_lmax(const Problem& P, int quirk) {
  double ke[576];
  canonical_stiffness(P.dx, P.dy, P.dz, P.nu, ke);
  return smoother_bound(ke, quirk);
}

template <typename T>
void configure_mg(MG<T>& mg, const Problem& P, const hexa_solve_params& prm) {
  mg.quirk = prm.diag_quirk;
  const double lmax = smoother_lmax(P, prm.diag_quirk);
  mg.smoother = prm.smoother;
  mg.omega = (T)(prm.jacobi_omega > 0 ? prm.jacobi_omega : 1.2 / lmax);
  mg.nu1 = prm.pre_smooth > 0 ? prm.pre_smooth : 1;
  mg.nu2 = prm.post_smooth >= 0 ? prm.post_smooth : 2;
  mg.citers = prm.coarse_iters >= 0 ? prm.coarse_iters : 30;
  mg.gamma = prm.mg_cycle == 2 ? 2 : 1;
  mg.set_chebyshev(lmax, std::max(mg.nu1, mg.nu2) + 1, prm.cheb_ratio > 1 ? prm.cheb_ratio : 10.0);
  mg.ke.assign(576, 0.0);
  if (canonical_stiffness(P.dx, P.dy, P.dz, P.nu, mg.ke.data()) != 0) mg.ke.clear();
}

bool setup_common(Ctx& c, const Problem& P, const hexa_solve_params& prm, ModalK<double>* K64, double* max_diag,
                  double* bnorm) {
  std::string e;
  if (!build_modal(P.dx, P.dy, P.dz, P.nu, K64, &e)) return c.fail(e);
  const long long n = P.g.ndof();
  double* diag = c.vec<double>("diag64", n);
  if (!diag) return false;
  const long long maxblocks = op_num_blocks<double>(P.g, pick_kchunk<double>(P.g)) + 8;
  if (!c.ensure_partials((size_t)std::max<long long>(maxblocks * 2, kRedBlocks * 2 + 16) + 4096)) return false;
  launch_diag<double>(P.g, P.m, P.fac64, *K64, prm.diag_quirk, 0.0, diag, nullptr, c.st);
  launch_max(diag, n, red(c, FIN_STORE, 1, nullptr, c.dscal + 0), kRedBlocks, c.st);
  c.launches += 2;
  launch_dot<double>(P.f64, P.f64, (const double*)nullptr, (const double*)nullptr, n,
                     red(c, FIN_STORE, 1, nullptr, c.dscal + 1), kRedBlocks, nullptr, c.st);
  c.launches++;
  cudaMemcpyAsync(c.hscal, c.dscal, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess) return c.cuda_ok("setup");
  *max_diag = c.hscal[0];
  *bnorm = std::sqrt(std::fmax(c.hscal[1], 0.0));
  return true;
}

template <typename T>
int solve_plain(Ctx& c, const Problem& P, const hexa_solve_params& prm, const double* u0, double* u,
                hexa_solve_stats* st) {
  const long long n = P.g.ndof();
  ModalK<double> K64;
  double max_diag = 0, bnorm = 0;
  cudaEventRecord(c.ev[0], c.st);
  if (!setup_common(c, P, prm, &K64, &max_diag, &bnorm)) return c.err.empty() ? HEXA_ERR_CUDA : HEXA_ERR_NOMEM;
  st->max_diag = max_diag;
  if (std::isnan(max_diag) || std::isinf(max_diag)) {  // GPUSolver.jl:310-315
    c.err = "Stiffness Matrix Diagonal contains NaN/Inf";
    cudaMemsetAsync(u, 0, sizeof(double) * n, c.st);
    st->relres = NAN;
    return HEXA_ERR_CORRUPT_INPUT;
  }
  if (bnorm == 0.0) {
    cudaMemsetAsync(u, 0, sizeof(double) * n, c.st);
    st->relres = 0.0;
    st->true_relres = 0.0;
    return HEXA_OK;
  }
  ModalK<T> K;
  if (Is64<T>::v) std::memcpy(&K, &K64, sizeof(K));
  else {
    ModalK<float> kf = modal_to_f32(K64);
    std::memcpy(&K, &kf, sizeof(K));
  }
  const T* fac = Host<T>::fac(c, P);
  const T* b;
  if (Is64<T>::v) b = (const T*)P.f64;
  else {
    T* bb = c.vec<T>("b_T", n);
    if (!bb) return HEXA_ERR_NOMEM;
    launch_convert<T, double>(bb, P.f64, n, c.st);
    c.launches++;
    b = bb;
  }
  Lev<T> L0;
  L0.g = P.g;
  L0.m = P.m;
  L0.fac = const_cast<T*>(fac);
  L0.kchunk = pick_kchunk<T>(P.g);
  PcgEnv<T> E;
  E.K = K;
  E.quirk = prm.diag_quirk;
  E.n = n;
  E.x = c.vec<T>("x_T", n);
  E.r = c.vec<T>("r_T", n);
  E.zA = c.vec<T>("zA_T", n);
  E.zB = c.vec<T>("zB_T", n);
  E.p = c.vec<T>("p_T", n);
  E.q = c.vec<T>("q_T", n);
  E.dinv = c.vec<T>("dinv_T", n);
  E.bestx = c.vec<T>("best_T", n);
  E.b = b;
  E.use_graphs = prm.use_graphs != 0;
  E.graph_iters = prm.graph_iters > 0 ? prm.graph_iters : 10;
  if (!fac || !E.x || !E.r || !E.zA || !E.zB || !E.p || !E.q || !E.dinv || !E.bestx) return HEXA_ERR_NOMEM;
  launch_fill<T>(E.bestx, T(0), n, c.st);  // best_x starts at zero (GPUSolver.jl:319)
  c.launches++;
  MG<T> mg;
  const bool want_mg = prm.precond == HEXA_PRECOND_MULTIGRID;
  int nlev = 1;
  if (want_mg) {
    nlev = plan_levels(P.g, prm.mg_levels);
    mg.K = K;
    configure_mg<T>(mg, P, prm);
    if (!build_mg<T>(c, mg, P.g, P.m, fac, nlev, std::string(Is64<T>::v ? "mg64_" : "mg32_"))) return HEXA_ERR_NOMEM;
    mg.L[0].kchunk = L0.kchunk;
  }
  if (!c.cuda_ok("solve setup")) return HEXA_ERR_CUDA;
  cudaEventRecord(c.ev[1], c.st);

  bool use_mg = want_mg;
  bool success = false;
  PcgOut last;
  double final_rel = 0.0, sigma = 0.0;
  int attempts = 0, total_iters = 0;
  double applies = 0.0;
  while (true) {
    double cur_shift = prm.shift_factor;
    bool fallback = false;
    for (int attempt = 1; attempt <= std::max(1, prm.max_shift_attempts); ++attempt) {
      ++attempts;
      sigma = cur_shift * max_diag;
      L0.sigma = (T)sigma;
      E.L0 = use_mg ? &mg.L[0] : &L0;
      E.mg = use_mg ? &mg : nullptr;
      bool x_zero = true;
      if (u0 && attempt == 1 && use_mg == want_mg) {
        launch_mask_copy<T, double>(P.g, P.m, E.x, u0, c.st);
        c.launches++;
        x_zero = false;
      } else {
        launch_fill<T>(E.x, T(0), n, c.st);
        c.launches++;
      }
      if (use_mg) mg_set_shift<T>(c, mg, sigma);
      else {
        launch_diag<T>(P.g, P.m, fac, K, prm.diag_quirk, (T)sigma, nullptr, E.dinv, c.st);
        c.launches++;
      }
      PcgOut o;
      if (!run_pcg<T>(c, E, prm.tol, prm.max_iter, prm.check_cadence, x_zero, bnorm, prm.divergence_check != 0, &o))
        return HEXA_ERR_CUDA;
      // FP64 true-residual restarts (plain FP64 only)
      if (o.status == 1 && prm.true_residual && Is64<T>::v) {
        double* r64 = c.vec<double>("rtrue", n);
        for (int rs = 0; rs < 4; ++rs) {
          const double tr = true_residual_norm(c, P, K64, prm.diag_quirk, sigma, (const double*)E.x, r64) / bnorm;
          applies += 1.0;
          if (tr <= prm.tol) break;
          PcgOut o2;
          const int left = prm.max_iter - o.iters;
          if (left <= 0) break;
          if (!run_pcg<T>(c, E, prm.tol, left, prm.check_cadence, false, bnorm, prm.divergence_check != 0, &o2))
            return HEXA_ERR_CUDA;
          o.iters += o2.iters;
          o.fine_applies += o2.fine_applies;
          o.status = o2.status;
          o.relres = o2.relres;
          if (o2.status != 1) break;
        }
      }
      last = o;
      total_iters += o.iters;
      applies += o.fine_applies;
      final_rel = o.relres;
      if (o.status == 1) {
        success = true;
        break;
      }
      const bool bad = (o.status == 2 || o.status == 3);
      if (bad && use_mg) {
        fallback = true;
        break;
      }
      if (bad && attempt < prm.max_shift_attempts) {
        cur_shift *= prm.shift_multiplier;
        continue;
      }
      if (prm.stagnation_tol > 0.0 && o.best_rel < prm.stagnation_tol) {
        cudaMemcpyAsync(E.x, E.bestx, sizeof(T) * n, cudaMemcpyDeviceToDevice, c.st);
        success = true;
        break;
      }
      cur_shift *= prm.shift_multiplier;
    }
    if (fallback) {
      use_mg = false;
      continue;
    }
    if (!success) cudaMemcpyAsync(E.x, E.bestx, sizeof(T) * n, cudaMemcpyDeviceToDevice, c.st);
    break;
  }
  if (Is64<T>::v) cudaMemcpyAsync(u, E.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.st);
  else {
    launch_convert<double, T>(u, E.x, n, c.st);
    c.launches++;
  }
  double* r64 = c.vec<double>("rtrue", n);
  const double tr = true_residual_norm(c, P, K64, prm.diag_quirk, sigma, u, r64) / bnorm;
  cudaEventRecord(c.ev[2], c.st);
  st->compliance = device_dot(c, P.f64, u, n, 9);
  cudaEventSynchronize(c.ev[2]);
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, c.ev[0], c.ev[1]);
  cudaEventElapsedTime(&ms2, c.ev[1], c.ev[2]);
  st->setup_ms = ms1;
  st->solve_ms = ms2;
  st->iterations = total_iters;
  st->attempts = attempts;
  st->relres = final_rel;
  st->true_relres = tr;
  st->shift = sigma;
  st->precond_used = use_mg ? HEXA_PRECOND_USED_MULTIGRID : HEXA_PRECOND_USED_JACOBI;
  st->mg_levels = use_mg ? (int)mg.L.size() : 1;
  st->smooth_steps = use_mg ? mg.nu2 : 0;
  st->fine_applies = applies;
  st->fine_applies_fp64 = Is64<T>::v ? applies : 1.0;
  if (!c.cuda_ok("solve")) return HEXA_ERR_CUDA;
  (void)last;
  return success ? HEXA_OK : HEXA_NOT_CONVERGED;
}

// Autotuner of the mixed form's multigrid: short FP32 GMG-PCG trials (120
// iterations, the rate measured over the last 60) on b = f/||f|| pick the level count (stage 1), the Chebyshev
// smoothing steps per side (stage 2) and the lower end lmax/ratio of the
// Chebyshev interval (stage 3) that minimise the estimated time to the
// tolerance, (log10(1/tol) / digits gained per iteration) * device time per
// iteration.  The choice is cached in the context per grid.
Ctx::Tuned autotune_mixed(Ctx& c, const Problem& P, const hexa_solve_params& prm, float* fac32,
                          const ModalK<float>& K32, double sigma, PcgEnv<float>& E, float* b32, double bnorm,
                          MG<float>& mg, bool search_ratio = false) {
  char key[128];
  std::snprintf(key, sizeof(key), "%d,%d,%d,%d,%g,%g,%g,%d", P.g.nx, P.g.ny, P.g.nz, prm.diag_quirk, P.nu, prm.tol,
                prm.shift_factor, search_ratio ? 1 : 0);
  auto it = c.tuned.find(key);
  if (it != c.tuned.end()) return it->second;
  const long long n = P.g.ndof();
  c.hscal[12] = 1.0 / bnorm;
  cudaMemcpyAsync(c.dscal + 12, c.hscal + 12, sizeof(double), cudaMemcpyHostToDevice, c.st);
  launch_scale_to_f32(b32, P.f64, c.dscal + 12, n, c.st);
  c.launches++;
  const double digits = std::log10(1.0 / prm.tol);
  const int lmax = plan_levels(P.g, 16);
  const int trial_iters = 120;
  auto trial = [&](int levels, int nu, int ratio) -> double {
    hexa_solve_params q = prm;
    q.pre_smooth = q.post_smooth = nu;
    q.cheb_ratio = ratio;
    mg = MG<float>();
    mg.K = K32;
    configure_mg<float>(mg, P, q);
    if (!build_mg<float>(c, mg, P.g, P.m, fac32, levels, "mg32_")) return INFINITY;
    mg_set_shift<float>(c, mg, sigma);
    E.L0 = &mg.L[0];
    E.mg = &mg;
    E.b = b32;
    launch_fill<float>(E.x, 0.0f, n, c.st);
    c.launches++;
    // the rate is taken over the second half of the trial, past the quickly
    // damped start, so that it reflects the slow modes that set the count
    PcgOut o;
    double ms = 0.0;
    if (!run_pcg<float>(c, E, 1e-30, trial_iters / 2, 1, true, 1.0, false, &o, &ms) || o.iters < 2) return INFINITY;
    const double rel_half = o.relres;
    PcgScalars h = *c.hs;
    h.max_iter = trial_iters;
    h.halt = 0;
    h.status = 0;
    *c.hs = h;
    cudaMemcpyAsync(c.s, c.hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, c.st);
    Graph g2;
    if (!pcg_drive<float>(c, E, g2, &h, &ms)) return INFINITY;
    const int iters = h.iter - o.iters;
    const double rel = h.relres;
    if (iters < 2 || !(rel > 0.0) || !(rel_half > 0.0) || !(rel < rel_half) || !(rel_half < 1.0)) return INFINITY;
    const double per_digit = iters / std::log10(rel_half / rel);
    return digits * per_digit * (ms / h.iter);
  };
  const int r0 = prm.cheb_ratio > 1 ? prm.cheb_ratio : 10;
  int best_l = std::max(2, lmax), best_nu = 3, best_r = r0;
  double best = INFINITY;
  for (int l = std::max(2, lmax - 2); l <= lmax; ++l) {
    const double t = trial(l, 3, r0);
    if (t < best) best = t, best_l = l;
  }
  for (int nu : {2, 4, 5}) {
    const double t = trial(best_l, nu, r0);
    if (t < best) best = t, best_nu = nu;
  }
  // The lower end of the Chebyshev interval (lambda_max / ratio) stays the
  // caller's for single solves: a short trial does not predict its effect on
  // the full count.  On the 384x192x192 cantilever with 7 levels and V(3,3),
  // whole solves took 4421 iterations at ratio 10 against 5173 at 5 and 5381
  // at 30, and a solve whose 120-iteration trials had picked a ratio other
  // than 10 took 6116 where ratio 10 takes 3996.  The block solve keeps the
  // search: on 8 load cases of the 256x128x128 cantilever it took 1264 block
  // iterations with the searched ratio and 1387 with ratio 10.
  if (search_ratio)
    for (int r : {5, 10, 20, 40}) {
      if (r == r0) continue;
      const double t = trial(best_l, best_nu, r);
      if (t < best) best = t, best_r = r;
    }
  Ctx::Tuned tu;
  tu.a = best_l;
  tu.b = best_nu;
  tu.c = best_r;
  c.tuned[key] = tu;
  return tu;
}

// Mixed precision: FP64 iterative refinement around FP32 GMG-PCG correction
// solves.  Each step rescales the FP64 residual to unit norm before it is
// rounded to FP32, so the 1e-9 contrast of void elements never meets FP32's
// range limits, and adds the correction back in FP64.
int solve_mixed(Ctx& c, const Problem& P, const hexa_solve_params& prm, const double* u0, double* u,
                hexa_solve_stats* st) {
  const long long n = P.g.ndof();
  ModalK<double> K64;
  double max_diag = 0, bnorm = 0;
  cudaEventRecord(c.ev[0], c.st);
  if (!setup_common(c, P, prm, &K64, &max_diag, &bnorm)) return c.err.empty() ? HEXA_ERR_CUDA : HEXA_ERR_NOMEM;
  st->max_diag = max_diag;
  if (std::isnan(max_diag) || std::isinf(max_diag)) {
    c.err = "Stiffness Matrix Diagonal contains NaN/Inf";
    cudaMemsetAsync(u, 0, sizeof(double) * n, c.st);
    st->relres = NAN;
    return HEXA_ERR_CORRUPT_INPUT;
  }
  if (bnorm == 0.0) {
    cudaMemsetAsync(u, 0, sizeof(double) * n, c.st);
    return HEXA_OK;
  }
  const double sigma = prm.shift_factor * max_diag;
  ModalK<float> K32 = modal_to_f32(K64);
  float* fac32 = c.vec<float>("fac_T", P.g.nelem());
  if (!fac32) return HEXA_ERR_NOMEM;
  launch_convert<float, double>(fac32, P.fac64, P.g.nelem(), c.st);
  c.launches++;
  Lev<float> L0;
  L0.g = P.g;
  L0.m = P.m;
  L0.fac = fac32;
  L0.kchunk = pick_kchunk<float>(P.g);
  L0.sigma = (float)sigma;
  PcgEnv<float> E;
  E.K = K32;
  E.quirk = prm.diag_quirk;
  E.n = n;
  E.x = c.vec<float>("x_T", n);
  E.r = c.vec<float>("r_T", n);
  E.zA = c.vec<float>("zA_T", n);
  E.zB = c.vec<float>("zB_T", n);
  E.p = c.vec<float>("p_T", n);
  E.q = c.vec<float>("q_T", n);
  E.dinv = c.vec<float>("dinv_T", n);
  float* b32 = c.vec<float>("b_T", n);
  double* r64 = c.vec<double>("rtrue", n);
  E.b = b32;
  E.use_graphs = prm.use_graphs != 0;
  E.graph_iters = prm.graph_iters > 0 ? prm.graph_iters : 10;
  if (!E.x || !E.r || !E.zA || !E.zB || !E.p || !E.q || !E.dinv || !b32 || !r64) return HEXA_ERR_NOMEM;
  MG<float> mg;
  const bool use_mg = prm.precond == HEXA_PRECOND_MULTIGRID;
  hexa_solve_params prm2 = prm;
  if (use_mg && prm.autotune) {
    const Ctx::Tuned t = autotune_mixed(c, P, prm, fac32, K32, sigma, E, b32, bnorm, mg);
    prm2.mg_levels = t.a;
    prm2.pre_smooth = prm2.post_smooth = t.b;
    prm2.cheb_ratio = t.c;
  }
  if (use_mg) {
    const int nlev = plan_levels(P.g, prm2.mg_levels);
    mg = MG<float>();
    mg.K = K32;
    configure_mg<float>(mg, P, prm2);
    if (!build_mg<float>(c, mg, P.g, P.m, fac32, nlev, "mg32_")) return HEXA_ERR_NOMEM;
    mg.L[0].kchunk = L0.kchunk;
    mg_set_shift<float>(c, mg, sigma);
    E.L0 = &mg.L[0];
    E.mg = &mg;
  } else {
    launch_diag<float>(P.g, P.m, fac32, K32, prm.diag_quirk, (float)sigma, nullptr, E.dinv, c.st);
    c.launches++;
    E.L0 = &L0;
  }
  if (u0) {
    launch_mask_copy<double, double>(P.g, P.m, u, u0, c.st);
  } else {
    launch_fill<double>(u, 0.0, n, c.st);
  }
  c.launches++;
  if (!c.cuda_ok("mixed setup")) return HEXA_ERR_CUDA;
  cudaEventRecord(c.ev[1], c.st);
  // One FP32 PCG carried across "reliable updates": the correction x32 is
  // accumulated into the FP64 iterate whenever the FP32 recursive residual has
  // dropped by inner_tol, the FP64 true residual f - (K + sigma I) u replaces
  // the FP32 residual (rescaled to unit norm, so void-contrast magnitudes never
  // meet FP32's range limits) and the search direction is kept, rescaled --
  // no restart, so the FP32 solve keeps its Krylov progress.
  double rn = true_residual_norm(c, P, K64, prm.diag_quirk, sigma, u, r64);
  double rel = rn / bnorm;
  double applies64 = 1.0, applies32 = 0.0;
  int outer = 0, status = HEXA_OK;
  const int max_outer = prm.max_outer > 0 ? prm.max_outer : 20;
  const double inner_tol = prm.inner_tol > 0 ? prm.inner_tol : 1e-4;
  double scale = 1.0 / rn;  // r32 = scale * r_true
  PcgScalars h;
  std::memset(&h, 0, sizeof(h));
  Graph graph;
  if (rel > prm.tol) {
    c.hscal[10] = scale;
    cudaMemcpyAsync(c.dscal + 10, c.hscal + 10, sizeof(double), cudaMemcpyHostToDevice, c.st);
    launch_scale_to_f32(b32, r64, c.dscal + 10, n, c.st);
    launch_fill<float>(E.x, 0.0f, n, c.st);
    c.launches += 2;
    h.tol = inner_tol;
    h.max_iter = prm.max_iter;
    h.cadence = prm.check_cadence;
    h.bnorm = 1.0;
    h.best_rel = INFINITY;
    h.no_div = 1;
    *c.hs = h;
    cudaMemcpyAsync(c.s, c.hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, c.st);
    const int* halt = &c.s->halt;
    launch_copy<float>(E.r, b32, n, c.st);
    c.launches++;
    if (E.mg) {
      vcycle<float>(c, *E.mg, 0, E.r, E.zA, halt);
      launch_dot<float>(E.r, E.zA, (const float*)nullptr, (const float*)nullptr, n, red(c, FIN_INIT_RZ, 1, c.s),
                        kRedBlocks, halt, c.st);
    } else {
      launch_jacobi_precond<float>(E.zA, E.r, E.dinv, n, red(c, FIN_INIT_RZ, 1, c.s), kRedBlocks, halt, c.st);
    }
    launch_copy<float>(E.p, E.zA, n, c.st);
    c.launches += 2;
    if (!c.cuda_ok("mixed setup")) return HEXA_ERR_CUDA;
  }
  while (rel > prm.tol) {
    if (!pcg_drive<float>(c, E, graph, &h)) return HEXA_ERR_CUDA;
    ++outer;
    if (h.status == 2) {  // NaN in the FP32 recursion
      status = HEXA_NOT_CONVERGED;
      break;
    }
    // accumulate the FP32 correction and recompute the true residual in FP64
    launch_add_scaled_f32(u, E.x, c.dscal + 10, n, c.st);
    c.launches++;
    rn = true_residual_norm(c, P, K64, prm.diag_quirk, sigma, u, r64);
    applies64 += 1.0;
    rel = rn / bnorm;
    if (rel <= prm.tol) break;
    if (h.iter >= prm.max_iter || outer >= max_outer || !(rel == rel)) {
      status = HEXA_NOT_CONVERGED;
      break;
    }
    // replace the residual, keep the direction: p <- z_new + beta * (scale_new/scale) p
    const double scale_new = 1.0 / rn, ratio = scale_new / scale;
    const double rz_old = h.rz * ratio * ratio;
    c.hscal[10] = scale_new;
    cudaMemcpyAsync(c.dscal + 10, c.hscal + 10, sizeof(double), cudaMemcpyHostToDevice, c.st);
    launch_scale_to_f32(E.r, r64, c.dscal + 10, n, c.st);
    launch_fill<float>(E.x, 0.0f, n, c.st);
    c.launches += 2;
    h.halt = 0;
    h.status = 0;
    h.best_rel = INFINITY;
    *c.hs = h;
    cudaMemcpyAsync(c.s, c.hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, c.st);
    const int* halt = &c.s->halt;
    if (E.mg) {
      vcycle<float>(c, *E.mg, 0, E.r, E.zA, halt);
      launch_dot<float>(E.r, E.zA, (const float*)nullptr, (const float*)nullptr, n, red(c, FIN_INIT_RZ, 1, c.s),
                        kRedBlocks, halt, c.st);
    } else {
      launch_jacobi_precond<float>(E.zA, E.r, E.dinv, n, red(c, FIN_INIT_RZ, 1, c.s), kRedBlocks, halt, c.st);
    }
    c.launches++;
    double rz_new = 0.0;
    cudaMemcpyAsync(c.hscal + 11, &c.s->rz, sizeof(double), cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess) {
      c.cuda_ok("reliable update");
      return HEXA_ERR_CUDA;
    }
    rz_new = c.hscal[11];
    const double beta = (rz_old > 0.0) ? rz_new / rz_old : 0.0;
    launch_axpby<float>(E.p, (float)(beta * ratio), E.zA, 1.0f, n, c.st);
    c.launches++;
    scale = scale_new;
  }
  applies32 = applies_per_iteration(E) * h.iter;
  const int inner_total = h.iter;
  cudaEventRecord(c.ev[2], c.st);
  st->compliance = device_dot(c, P.f64, u, n, 9);
  cudaEventSynchronize(c.ev[2]);
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, c.ev[0], c.ev[1]);
  cudaEventElapsedTime(&ms2, c.ev[1], c.ev[2]);
  st->setup_ms = ms1;
  st->solve_ms = ms2;
  st->iterations = inner_total;
  st->outer_iterations = outer;
  st->attempts = 1;
  st->relres = rel;
  st->true_relres = rel;
  st->shift = sigma;
  st->precond_used = use_mg ? HEXA_PRECOND_USED_MULTIGRID : HEXA_PRECOND_USED_JACOBI;
  st->mg_levels = use_mg ? (int)mg.L.size() : 1;
  st->smooth_steps = use_mg ? mg.nu2 : 0;
  st->fine_applies = applies32 + applies64;
  st->fine_applies_fp64 = applies64;
  if (!c.cuda_ok("mixed solve")) return HEXA_ERR_CUDA;
  return status;
}

// k load cases as one block PCG (block.cu) on the columns of F (k <= 16).
// T = float: FP32 operator, V-cycles and block recursion, carried across
// reliable updates -- whenever every active column's recursive residual has
// dropped by inner_tol, the FP32 corrections are added to the FP64 iterate
// U, the FP64 true residuals F - (K + sigma I) U replace the FP32 residuals
// (each rescaled to unit norm) and the iteration continues with its search
// directions, which the block A-orthogonalisation keeps valid.  A column
// whose true relative residual meets tol is frozen (its scale set to 0: zero
// residual, no further correction).  T = double: the same loop in FP64.
template <typename T>
int solve_block(Ctx& c, const Problem& P, int k, const hexa_solve_params& prm, double* U, hexa_solve_stats* st) {
  const long long n = P.g.ndof();
  ModalK<double> K64;
  double max_diag = 0, f0norm = 0;
  cudaEventRecord(c.ev[0], c.st);
  if (!setup_common(c, P, prm, &K64, &max_diag, &f0norm)) return c.err.empty() ? HEXA_ERR_CUDA : HEXA_ERR_NOMEM;
  st->max_diag = max_diag;
  if (std::isnan(max_diag) || std::isinf(max_diag)) {
    c.err = "Stiffness Matrix Diagonal contains NaN/Inf";
    cudaMemsetAsync(U, 0, sizeof(double) * n * k, c.st);
    st->relres = NAN;
    return HEXA_ERR_CORRUPT_INPUT;
  }
  const double sigma = prm.shift_factor * max_diag;
  const int kc = block_kc(k);
  if (!c.ensure_partials((size_t)block_partials_needed(k) + 4096)) return HEXA_ERR_NOMEM;
  ModalK<T> K;
  if (Is64<T>::v) std::memcpy(&K, &K64, sizeof(K));
  else {
    ModalK<float> kf = modal_to_f32(K64);
    std::memcpy(&K, &kf, sizeof(K));
  }
  const T* fac = Host<T>::fac(c, P);
  T* X = c.vec<T>("blk_X", n * k);
  T* R = c.vec<T>("blk_R", n * k);
  T* Z = c.vec<T>("blk_Z", n * k);
  T* Pd = c.vec<T>("blk_P", n * k);
  T* Q = c.vec<T>("blk_Q", n * k);
  T* dinv = c.vec<T>("blk_dinv", n);
  double* R64 = c.vec<double>("blk_R64", n * k);
  // small arrays: gram1 (kc x 2kc), gram2 (kc x kc), alpha, beta (k x k),
  // column norms, scales
  double* sm = c.vec<double>("blk_small", 4096);
  if (!fac || !X || !R || !Z || !Pd || !Q || !dinv || !R64 || !sm) return HEXA_ERR_NOMEM;
  double *gram1 = sm, *gram2 = sm + 1024, *alpha = sm + 1536, *beta = sm + 1792, *rr = sm + 2048,
         *fn2 = sm + 2080, *rn2 = sm + 2112, *scale = sm + 2144, *comp = sm + 2176;
  double* hsm = c.hscal;  // 64 pinned doubles: [0,k) norms, [16, 16+k) scales
  unsigned* gticket = c.ticket + 32;
  cudaMemsetAsync(gticket, 0, sizeof(unsigned), c.st);
  // column norms of F
  {
    RedArgs r = red(c, FIN_STORE, 1, nullptr, fn2);
    r.ncol = k;
    launch_dot<double>(P.f64, P.f64, (const double*)nullptr, (const double*)nullptr, n, r, kRedBlocks * k, nullptr,
                       c.st);
    c.launches++;
  }
  cudaMemcpyAsync(hsm, fn2, sizeof(double) * k, cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess) return c.cuda_ok("block setup") ? HEXA_ERR_CUDA : HEXA_ERR_CUDA;
  std::vector<double> fnorm(k);
  for (int j = 0; j < k; ++j) fnorm[j] = std::sqrt(std::fmax(hsm[j], 0.0));

  Lev<T> L0;
  L0.g = P.g;
  L0.m = P.m;
  L0.fac = const_cast<T*>(fac);
  L0.kchunk = pick_kchunk<T>(P.g);
  L0.sigma = (T)sigma;
  MG<T> mg;
  const bool use_mg = prm.precond == HEXA_PRECOND_MULTIGRID;
  if (use_mg) {
    hexa_solve_params prm2 = prm;
    if constexpr (!Is64<T>::v) {
      // the single-grid autotuner (cached per grid), run on the first loaded column
      int j0 = 0;
      while (j0 < k - 1 && !(fnorm[j0] > 0)) ++j0;
      if (prm.autotune && fnorm[j0] > 0) {
        Problem P0 = P;
        P0.f64 = P.f64 + (long long)j0 * n;
        PcgEnv<float> E;
        E.K = K;
        E.quirk = prm.diag_quirk;
        E.n = n;
        E.x = X;
        E.r = R;
        E.zA = Z;
        E.zB = Q;
        E.p = Pd;
        E.q = Q + n * (k > 1 ? 1 : 0);
        E.dinv = dinv;
        E.use_graphs = prm.use_graphs != 0;
        E.graph_iters = prm.graph_iters > 0 ? prm.graph_iters : 10;
        float* b32 = c.vec<float>("blk_tune_b", n);
        float* qbuf = k > 1 ? nullptr : c.vec<float>("blk_tune_q", n);
        if (!b32 || (k == 1 && !qbuf)) return HEXA_ERR_NOMEM;
        if (k == 1) E.q = qbuf;
        MG<float> tmg;
        const Ctx::Tuned t =
            autotune_mixed(c, P0, prm, const_cast<float*>(fac), K, sigma, E, b32, fnorm[j0], tmg, true);
        prm2.mg_levels = t.a;
        prm2.pre_smooth = prm2.post_smooth = t.b;
        prm2.cheb_ratio = t.c;
      }
    }
    mg.K = K;
    configure_mg<T>(mg, P, prm2);
    if (!build_mg<T>(c, mg, P.g, P.m, fac, plan_levels(P.g, prm2.mg_levels),
                     std::string(Is64<T>::v ? "mg64_" : "mg32_")))
      return HEXA_ERR_NOMEM;
    mg.L[0].kchunk = L0.kchunk;
    mg_set_shift<T>(c, mg, sigma);
  } else {
    launch_diag<T>(P.g, P.m, fac, K, prm.diag_quirk, (T)sigma, nullptr, dinv, c.st);
    c.launches++;
  }
  Lev<T>& LA = use_mg ? mg.L[0] : L0;
  Lev<double> L64;
  L64.g = P.g;
  L64.m = P.m;
  L64.fac = const_cast<double*>(P.fac64);
  L64.sigma = sigma;
  L64.kchunk = pick_kchunk<double>(P.g);

  // start: U = 0, P = Q = 0, G = identity (so the first beta is zero)
  launch_fill<double>(U, 0.0, n * k, c.st);
  launch_fill<T>(Pd, T(0), n * k, c.st);
  launch_fill<T>(Q, T(0), n * k, c.st);
  launch_fill<double>(gram1, 0.0, 1024, c.st);
  c.launches += 4;
  {
    std::vector<double> id((size_t)kc * 2 * kc, 0.0);
    for (int j = 0; j < kc; ++j) id[(size_t)j * 2 * kc + j] = 1.0;
    cudaMemcpyAsync(gram1, id.data(), id.size() * sizeof(double), cudaMemcpyHostToDevice, c.st);
    cudaStreamSynchronize(c.st);
  }
  const int* halt = &c.s->halt;
  const double eps = Is64<T>::v ? 1e-12 : 1e-6;
  // k-column buffers of the block V-cycle (levels 1.. also need right-hand
  // sides and solutions); the W-cycle runs column by column
  ColBufs<T> cb;
  const bool cols = use_mg && mg.gamma == 1 && k > 1;
  if (cols) {
    const int nl = (int)mg.L.size();
    cb.xa.assign(nl, nullptr), cb.xb.assign(nl, nullptr), cb.b.assign(nl, nullptr), cb.r.assign(nl, nullptr);
    for (int l = 0; l < nl; ++l) {
      const long long nl_dof = mg.L[l].g.ndof() * (long long)k;
      const std::string s = "blkmg_" + std::to_string(l) + "_";
      if (l + 1 < nl) {
        cb.xb[l] = c.vec<T>(s + "xb", nl_dof);
        cb.r[l] = c.vec<T>(s + "r", nl_dof);
        if (!cb.xb[l] || !cb.r[l]) return HEXA_ERR_NOMEM;
      }
      if (l > 0) {
        cb.b[l] = c.vec<T>(s + "b", nl_dof);
        cb.xa[l] = c.vec<T>(s + "xa", nl_dof);
        if (!cb.b[l] || !cb.xa[l]) return HEXA_ERR_NOMEM;
      }
    }
  }
  auto iteration = [&]() {
    if (cols) {
      vcycle_cols<T>(c, mg, cb, 0, R, Z, k, halt);
    } else if (use_mg) {
      for (int j = 0; j < k; ++j) vcycle<T>(c, mg, 0, R + (long long)j * n, Z + (long long)j * n, halt);
    } else {
      launch_cols_jacobi<T>(Z, R, dinv, n, k, halt, c.st);
      c.launches++;
    }
    launch_gram<T>(Q, Z, (const T*)nullptr, k, n, c.partials, gticket, gram2, halt, c.st);
    launch_block_solve(gram1, 2 * kc, gram2, kc, 0, k, -1.0, eps, beta, halt, c.st);
    launch_block_p_update<T>(Pd, Z, beta, k, n, halt, c.st);
    OpArgs<T> a = opargs<T>(LA, K, prm.diag_quirk, Pd, nullptr, Q, T(0), halt, red(c, FIN_NONE, 1, nullptr));
    a.ncol = k;
    op<T>(c, OP_APPLY, a);
    launch_gram<T>(Pd, Q, R, k, n, c.partials, gticket, gram1, halt, c.st);
    launch_block_solve(gram1, 2 * kc, gram1, 2 * kc, kc, k, 1.0, eps, alpha, halt, c.st);
    RedArgs ru = red(c, FIN_BLOCK_RES, k, c.s, rr);
    launch_block_update<T>(X, R, Pd, Q, alpha, k, n, ru, c.st);
    c.launches += 6;
  };
  auto true_residuals = [&](std::vector<double>& rel) -> bool {
    OpArgs<double> a = opargs<double>(L64, K64, prm.diag_quirk, U, P.f64, R64, 0.0, nullptr, red(c, FIN_NONE, 1, nullptr));
    a.ncol = k;
    op<double>(c, OP_RESID, a);
    RedArgs r = red(c, FIN_STORE, 1, nullptr, rn2);
    r.ncol = k;
    launch_dot<double>(R64, R64, (const double*)nullptr, (const double*)nullptr, n, r, kRedBlocks * k, nullptr, c.st);
    c.launches++;
    cudaMemcpyAsync(hsm, rn2, sizeof(double) * k, cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess) return c.cuda_ok("block residual");
    for (int j = 0; j < k; ++j) rel[j] = fnorm[j] > 0 ? std::sqrt(std::fmax(hsm[j], 0.0)) / fnorm[j] : 0.0;
    return true;
  };
  if (!c.cuda_ok("block setup")) return HEXA_ERR_CUDA;
  cudaEventRecord(c.ev[1], c.st);

  std::vector<double> rel(k, 0.0);
  const double inner_tol = Is64<T>::v ? 0.0 : (prm.inner_tol > 0 ? prm.inner_tol : 1e-4);
  const int max_outer = prm.max_outer > 0 ? prm.max_outer : 20;
  int outer = 0, status = HEXA_OK, applies64 = 0;
  PcgScalars h;
  std::memset(&h, 0, sizeof(h));
  h.max_iter = prm.max_iter;
  h.bnorm = 1.0;
  h.best_rel = INFINITY;
  h.no_div = 1;
  Graph graph;
  int G = prm.graph_iters > 0 ? prm.graph_iters : 10;
  const bool graphs = prm.use_graphs != 0;
  double worst = 0.0;
  while (true) {
    if (!true_residuals(rel)) return HEXA_ERR_CUDA;
    ++applies64;
    worst = 0.0;
    for (int j = 0; j < k; ++j) worst = std::fmax(worst, rel[j]);
    if (!(worst == worst)) {
      status = HEXA_NOT_CONVERGED;
      break;
    }
    if (worst <= prm.tol) break;
    if (outer >= max_outer || h.iter >= prm.max_iter || h.status == 2) {
      status = HEXA_NOT_CONVERGED;
      break;
    }
    // rescale: active columns to unit norm, converged ones frozen
    double need = 1.0;  // scaled residual that brings every active column to tol
    for (int j = 0; j < k; ++j) {
      const double rn = rel[j] * fnorm[j];
      hsm[16 + j] = (rel[j] <= prm.tol || rn == 0.0) ? 0.0 : 1.0 / rn;
      if (hsm[16 + j] != 0.0) need = std::fmin(need, prm.tol / rel[j]);
    }
    cudaMemcpyAsync(scale, hsm + 16, sizeof(double) * k, cudaMemcpyHostToDevice, c.st);
    launch_cols_from64<T>(R, R64, scale, n, k, c.st);
    launch_fill<T>(X, T(0), n * k, c.st);
    c.launches += 2;
    // the FP64 recursion runs to the outer tolerance in one pass
    h.tol = Is64<T>::v ? 0.5 * need : std::fmax(inner_tol, 0.5 * need);
    h.halt = 0;
    h.status = 0;
    h.best_rel = INFINITY;
    *c.hs = h;
    cudaMemcpyAsync(c.s, c.hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, c.st);
    if (graphs && !graph.exec) {
      if (!capture(c, graph, [&]() {
            for (int i = 0; i < G; ++i) iteration();
          }))
        return HEXA_ERR_CUDA;
    }
    while (true) {
      if (graphs) {
        if (!replay(c, graph)) return HEXA_ERR_CUDA;
      } else {
        for (int i = 0; i < G; ++i) iteration();
      }
      cudaMemcpyAsync(c.hs, c.s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c.st);
      if (cudaStreamSynchronize(c.st) != cudaSuccess) return c.cuda_ok("block pcg") ? HEXA_ERR_CUDA : HEXA_ERR_CUDA;
      h = *c.hs;
      if (h.halt) break;
    }
    ++outer;
    launch_cols_accum<T>(U, X, scale, n, k, c.st);
    c.launches++;
  }
  // compliance: equal-weighted sum over the load cases of f_j . u_j
  {
    RedArgs r = red(c, FIN_STORE, 1, nullptr, comp);
    r.ncol = k;
    launch_dot<double>(P.f64, U, (const double*)nullptr, (const double*)nullptr, n, r, kRedBlocks * k, nullptr, c.st);
    c.launches++;
  }
  cudaMemcpyAsync(hsm, comp, sizeof(double) * k, cudaMemcpyDeviceToHost, c.st);
  cudaEventRecord(c.ev[2], c.st);
  cudaEventSynchronize(c.ev[2]);
  double compl_sum = 0.0;
  for (int j = 0; j < k; ++j) compl_sum += hsm[j];
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, c.ev[0], c.ev[1]);
  cudaEventElapsedTime(&ms2, c.ev[1], c.ev[2]);
  st->setup_ms = ms1;
  st->solve_ms = ms2;
  st->iterations = h.iter;
  st->outer_iterations = outer;
  st->attempts = 1;
  st->relres = worst;
  st->true_relres = worst;
  st->shift = sigma;
  st->compliance = compl_sum;
  st->precond_used = use_mg ? HEXA_PRECOND_USED_MULTIGRID : HEXA_PRECOND_USED_JACOBI;
  st->mg_levels = use_mg ? (int)mg.L.size() : 1;
  st->smooth_steps = use_mg ? mg.nu2 : 0;
  st->fine_applies = (applies_per_iteration_mg(use_mg ? &mg : nullptr)) * h.iter * k + applies64 * k;
  st->fine_applies_fp64 = Is64<T>::v ? st->fine_applies : (double)applies64 * k;
  if (!c.cuda_ok("block solve")) return HEXA_ERR_CUDA;
  return status;
}

// ||f - K u|| / ||f|| in FP64 without the diagonal shift: the residual of the
// unshifted system, which the shifted solve (GPUSolver.jl:343) leaves at about
// sigma ||u|| / ||f||.  Equal to the solve's own true residual when sigma = 0.
double unshifted_relres(Ctx& c, const Problem& P, int quirk, const double* u) {
  ModalK<double> K64;
  std::string e;
  if (!build_modal(P.dx, P.dy, P.dz, P.nu, &K64, &e)) return NAN;
  double* r64 = c.vec<double>("rtrue", P.g.ndof());
  if (!r64) return NAN;
  const double fnorm = std::sqrt(std::fmax(device_dot(c, P.f64, P.f64, P.g.ndof(), 13), 0.0));
  if (fnorm == 0.0) return 0.0;
  return true_residual_norm(c, P, K64, quirk, 0.0, u, r64) / fnorm;
}

}  // namespace

int solve_problem(Ctx& c, const Problem& P, const hexa_solve_params& prm, const double* u0, double* u,
                  hexa_solve_stats* st) {
  int rc;
  switch (prm.precision) {
    case HEXA_PREC_FP64: rc = solve_plain<double>(c, P, prm, u0, u, st); break;
    case HEXA_PREC_FP32: rc = solve_plain<float>(c, P, prm, u0, u, st); break;
    case HEXA_PREC_MIXED: rc = solve_mixed(c, P, prm, u0, u, st); break;
    default: c.err = "unknown precision"; return HEXA_ERR_ARG;
  }
  if (rc >= 0) st->unshifted_relres = (st->shift == 0.0) ? st->true_relres : unshifted_relres(c, P, prm.diag_quirk, u);
  return rc;
}

int multi_rhs_problem(Ctx& c, const Problem& P, int k, const double* F_dev, const hexa_solve_params& prm,
                      double* U_dev, hexa_solve_stats* st) {
  // groups of up to 16 columns, each one block PCG
  const long long n = P.g.ndof();
  hexa_solve_stats acc;
  std::memset(&acc, 0, sizeof(acc));
  int worst = HEXA_OK;
  for (int j0 = 0; j0 < k; j0 += kMaxBlockCols) {
    const int kb = std::min(kMaxBlockCols, k - j0);
    Problem Q = P;
    Q.f64 = F_dev + (long long)j0 * n;
    hexa_solve_stats s1;
    std::memset(&s1, 0, sizeof(s1));
    int rc = (prm.precision == HEXA_PREC_FP64) ? solve_block<double>(c, Q, kb, prm, U_dev + (long long)j0 * n, &s1)
                                              : solve_block<float>(c, Q, kb, prm, U_dev + (long long)j0 * n, &s1);
    if (rc < 0) return rc;
    if (rc > worst) worst = rc;
    acc.iterations += s1.iterations;
    acc.outer_iterations += s1.outer_iterations;
    acc.attempts = 1;
    acc.setup_ms += s1.setup_ms;
    acc.solve_ms += s1.solve_ms;
    acc.compliance += s1.compliance;
    acc.relres = std::fmax(acc.relres, s1.relres);
    acc.true_relres = std::fmax(acc.true_relres, s1.true_relres);
    acc.fine_applies += s1.fine_applies;
    acc.fine_applies_fp64 += s1.fine_applies_fp64;
    acc.precond_used = s1.precond_used;
    acc.mg_levels = s1.mg_levels;
    acc.smooth_steps = s1.smooth_steps;
    acc.shift = s1.shift;
    acc.max_diag = s1.max_diag;
    for (int j = 0; j < kb; ++j) {
      Problem Qj = P;
      Qj.f64 = F_dev + (long long)(j0 + j) * n;
      const double* uj = U_dev + (long long)(j0 + j) * n;
      const double ur = (s1.shift == 0.0 && kb == 1) ? s1.true_relres : unshifted_relres(c, Qj, prm.diag_quirk, uj);
      acc.unshifted_relres = std::fmax(acc.unshifted_relres, ur);
    }
  }
  *st = acc;
  return worst;
}

}  // namespace hexa
