// Batches of independent problems on grids of uneven sizes, solved together.
//
// Every kernel of a PCG iteration is ONE launch over all instances: each
// instance owns a block range of the launch and gets its own reductions,
// device scalars and halt flag (a converged instance's blocks return at
// once).  The operator launch is the persistent static-stride kernel of the
// single grid, its (tile, z-brick) items taken per instance.  The V-cycle
// runs level by level over the instances that have that level: an instance
// whose hierarchy ends at level l is solved there by the one-CTA coarse
// kernel (one CTA per instance) while the others smooth, restrict and
// recurse.  Groups of iterations replay from one CUDA graph.  With autotune
// on, the operator's z-brick depth is picked by timing the batched sweep.
//
// Solve: FP32 GMG-PCG per instance carried across reliable updates against
// FP64 true residuals (as the single-grid mixed path), converged instances
// frozen.  Filter: the Helmholtz filter's Jacobi-PCG per instance with the
// semantics of GPUHelmholtz.jl:190-266 (test every 10 iterations, cap).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "element.h"
#include "hexa_kernels.h"
#include "solver.h"

namespace hexa {

namespace {

constexpr int kBatchVecBlocks = 152 * 8;

struct DevTable {
  std::vector<BatchInst> h;
  BatchInst* d = nullptr;
  int oblocks = 0, vblocks = 0;
  int n() const { return (int)h.size(); }
};

bool upload(Ctx& c, DevTable& t, const std::string& name) {
  if (t.h.empty()) return true;
  t.d = c.vec<BatchInst>(name, t.h.size());
  if (!t.d) return false;
  cudaMemcpyAsync(t.d, t.h.data(), t.h.size() * sizeof(BatchInst), cudaMemcpyHostToDevice, c.st);
  return true;
}

struct BatchCtx {
  Ctx& c;
  int count;
  PcgScalars* s;     // per-instance scalars
  unsigned* ticket;  // per-instance tickets
};

RedArgs bred(const BatchCtx& B, int op, int nsum, double* dst = nullptr) {
  RedArgs r;
  r.partials = B.c.partials;
  r.ticket = B.ticket;
  r.dst = dst;
  r.s = B.s;
  r.op = op;
  r.nsum = nsum;
  return r;
}

template <typename T>
struct BLevel {
  std::vector<int> inst;  // instances that have this level
  std::vector<Grid> g;
  std::vector<long long> off, eoff;
  long long ndof = 0, nelem = 0;
  T *fac = nullptr, *xa = nullptr, *xb = nullptr, *b = nullptr, *r = nullptr;
  T *dinv = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *w = nullptr;  // coarse scratch
  DevTable smooth;   // instances that smooth here
  DevTable coarse;   // instances whose coarsest level this is
  DevTable restr;    // next-level instances: g = next level, g2 = this level
  DevTable prolong;  // smoothing instances: g = this level, g2 = next level
};

template <typename T>
struct BatchMG {
  std::vector<BLevel<T>> L;
  ModalK<T> K;
  int quirk = 0, nu1 = 2, nu2 = 2, citers = 30;
  bool cheb = true, idx32 = true;
  T omega = T(0.6), inv_theta = T(0);
  std::vector<T> c1, c2;
};

template <typename T>
BatchOpArgs<T> bop(const BatchCtx& B, const ModalK<T>& K, int quirk, const DevTable& t, const T* fac, const T* x,
                   const T* b, T* y, const T* xin, T c1, T c2, T omega, RedArgs red) {
  BatchOpArgs<T> a;
  a.K = K;
  a.c1 = c1;
  a.c2 = c2;
  a.omega = omega;
  a.diag_quirk = quirk;
  a.inst = t.d;
  a.ninst = t.n();
  a.nblocks = t.oblocks;
  a.x = x;
  a.fac = fac;
  a.b = b;
  a.y = y;
  a.xin = xin;
  a.red = red;
  a.s = B.s;
  return a;
}

template <typename T>
void bvcycle(BatchCtx& B, BatchMG<T>& mg, int l, const T* b, T* xout) {
  Ctx& c = B.c;
  BLevel<T>& V = mg.L[l];
  if (V.coarse.n()) {
    long long mnd = 0, mne = 0;
    for (const BatchInst& ci : V.coarse.h) mnd = std::max(mnd, ci.g.ndof()), mne = std::max(mne, ci.g.nelem());
    launch_batch_coarse_pcg<T>(V.coarse.d, V.coarse.n(), V.fac, mg.K, V.dinv, b, xout, V.r, V.z, V.p, V.q, V.w,
                               mg.citers, B.s, c.st, mnd, mne);
    c.launches++;
  }
  if (!V.smooth.n()) return;
  const int nw = mg.nu1 + mg.nu2;
  auto bufw = [&](int w) -> T* { return ((nw - 1 - w) % 2 == 0) ? xout : V.xb; };
  int w = 0;
  T* cur = bufw(w++);
  const RedArgs none = bred(B, FIN_NONE, 1);
  const T* prev = nullptr;
  auto op = [&](int mode, const T* x, T* y, const T* xin, T c1, T c2, T omega) {
    launch_op_batch<T>(mode, bop<T>(B, mg.K, mg.quirk, V.smooth, V.fac, x, b, y, xin, c1, c2, omega, none), mg.idx32,
                       c.st);
    c.launches++;
  };
  auto cheb_step = [&](int s) {
    T* nx = bufw(w++);
    op(OP_CHEB2, cur, nx, prev, mg.c1[s], mg.c2[s], T(0));
    prev = cur;
    cur = nx;
  };
  launch_batch_jacobi0<T>(V.smooth.d, V.smooth.n(), V.smooth.vblocks, V.fac, mg.K, mg.quirk,
                          mg.cheb ? mg.inv_theta : mg.omega, b, cur, B.s, c.st);
  c.launches++;
  for (int s = 1; s < mg.nu1; ++s) {
    if (mg.cheb) {
      cheb_step(s);
    } else {
      T* nx = bufw(w++);
      op(OP_JACOBI, cur, nx, nullptr, T(0), T(0), mg.omega);
      cur = nx;
    }
  }
  op(OP_RESID, cur, V.r, nullptr, T(0), T(0), T(0));
  BLevel<T>& C = mg.L[l + 1];
  launch_batch_restrict<T>(V.restr.d, V.restr.n(), V.restr.vblocks, V.r, C.b, B.s, c.st);
  c.launches++;
  bvcycle<T>(B, mg, l + 1, C.b, C.xa);
  launch_batch_prolong_add<T>(V.prolong.d, V.prolong.n(), V.prolong.vblocks, C.xa, cur, B.s, c.st);
  c.launches++;
  for (int s = 0; s < mg.nu2; ++s) {
    if (mg.cheb && s > 0) {
      cheb_step(s);
    } else {
      T* nx = bufw(w++);
      op(OP_JACOBI, cur, nx, nullptr, T(0), T(0), mg.cheb ? mg.inv_theta : mg.omega);
      prev = cur;
      cur = nx;
    }
  }
}

// Coarse grid of a batch level: every axis halved, an odd axis rounded up.
// The extra half element of a rounded axis lies past the fine grid's high
// face; its fine children do not exist, so it coarsens to a factor averaged
// over the children that do (a partly void element), restriction gathers
// only fine nodes that exist and prolongation never reads past the coarse
// grid.  For an even axis this is the plain 2:1 halving.
Grid batch_coarse_grid(const Grid& g) { return make_grid((g.nx + 1) / 2, (g.ny + 1) / 2, (g.nz + 1) / 2); }

// Coarsest grids of a batch are solved by one CTA's Jacobi-PCG each, whose
// time follows the largest of them, so batch hierarchies coarsen further
// than the single-grid one (whose dense coarsest solve wants ~2500 nodes).
constexpr long long kBatchCoarseNodes = 1000;

// Level count of one instance: halve (rounding an odd axis up) while every
// axis is >= 4, down to kBatchCoarseNodes nodes, or the requested count.  An
// odd axis whose high face is clamped stops coarsening: the rounded-up
// coarse grid would move that face half an element outwards.
int batch_levels(const Grid& g, uint32_t faces, int requested) {
  int nx = g.nx, ny = g.ny, nz = g.nz, lv = 1;
  const int maxlv = requested > 0 ? requested : 16;
  while (lv < maxlv) {
    if (nx < 4 || ny < 4 || nz < 4) break;
    if (((nx & 1) && (faces & 2u)) || ((ny & 1) && (faces & 8u)) || ((nz & 1) && (faces & 32u))) break;
    if (requested <= 0 && (long long)(nx + 1) * (ny + 1) * (nz + 1) <= kBatchCoarseNodes) break;
    nx = (nx + 1) / 2;
    ny = (ny + 1) / 2;
    nz = (nz + 1) / 2;
    ++lv;
  }
  return lv;
}

// Buffers, coarse factors, coarse diagonals and device tables of the batch
// hierarchy; the operator tables use z-bricks of kchunk layers.
template <typename T>
bool build_batch_mg(Ctx& c, BatchMG<T>& mg, const std::vector<Grid>& g0, const std::vector<uint32_t>& faces,
                    const std::vector<double>& sigma, const std::vector<int>& nlev, const T* fac0, int kchunk) {
  const int n = (int)g0.size();
  int maxlev = 0;
  for (int v : nlev) maxlev = std::max(maxlev, v);
  mg.L.assign(maxlev, BLevel<T>());
  const std::string tag = sizeof(T) == 8 ? "bmg64_" : "bmg32_";
  for (int l = 0; l < maxlev; ++l) {
    BLevel<T>& V = mg.L[l];
    for (int i = 0; i < n; ++i) {
      if (nlev[i] <= l) continue;
      Grid g = g0[i];
      for (int q = 0; q < l; ++q) g = batch_coarse_grid(g);
      V.inst.push_back(i);
      V.g.push_back(g);
      V.off.push_back(V.ndof);
      V.eoff.push_back(V.nelem);
      V.ndof += g.ndof();
      V.nelem += g.nelem();
    }
    const std::string s = tag + std::to_string(l);
    V.fac = l == 0 ? const_cast<T*>(fac0) : c.vec<T>(s + "fac", V.nelem);
    V.xb = c.vec<T>(s + "xb", V.ndof);
    V.r = c.vec<T>(s + "r", V.ndof);
    if (l > 0) {
      V.xa = c.vec<T>(s + "xa", V.ndof);
      V.b = c.vec<T>(s + "b", V.ndof);
    }
    if (!V.fac || !V.xb || !V.r || (l > 0 && (!V.xa || !V.b))) return false;
    for (size_t k = 0; k < V.inst.size(); ++k) {
      const int i = V.inst[k];
      BatchInst bi;
      std::memset(&bi, 0, sizeof(bi));
      bi.g = V.g[k];
      bi.m.faces = faces[i];
      bi.off = V.off[k];
      bi.noff = V.off[k] / 3;
      bi.eoff = V.eoff[k];
      bi.sigma = sigma[i] * std::pow(8.0, l);  // row sums of P^T P
      bi.id = i;
      if (nlev[i] - 1 == l) {
        V.coarse.h.push_back(bi);
      } else {
        V.smooth.h.push_back(bi);
        bi.g2 = batch_coarse_grid(bi.g);
        bi.m2.faces = faces[i];
        V.prolong.h.push_back(bi);  // off2 filled below
      }
    }
    if (V.coarse.n()) {
      V.dinv = c.vec<T>(s + "dinv", V.ndof);
      V.p = c.vec<T>(s + "p", V.ndof);
      V.q = c.vec<T>(s + "q", V.ndof);
      V.z = c.vec<T>(s + "z", V.ndof);
      V.w = c.vec<T>(s + "w", 24 * V.nelem);
      if (!V.dinv || !V.p || !V.q || !V.z || !V.w) return false;
    }
  }
  for (int l = 0; l + 1 < maxlev; ++l) {
    BLevel<T>& V = mg.L[l];
    BLevel<T>& C = mg.L[l + 1];
    for (size_t k = 0; k < C.inst.size(); ++k) {
      const int i = C.inst[k];
      const size_t kf = std::find(V.inst.begin(), V.inst.end(), i) - V.inst.begin();
      BatchInst bi;
      std::memset(&bi, 0, sizeof(bi));
      bi.g = C.g[k];
      bi.m.faces = faces[i];
      bi.off = C.off[k];
      bi.noff = C.off[k] / 3;
      bi.eoff = C.eoff[k];
      bi.g2 = V.g[kf];
      bi.m2.faces = faces[i];
      bi.off2 = V.off[kf];
      bi.id = i;
      V.restr.h.push_back(bi);
      launch_coarsen_factors<T>(V.g[kf], V.fac + V.eoff[kf], C.g[k], C.fac + C.eoff[k], c.st);
      c.launches++;
    }
    for (BatchInst& pr : V.prolong.h) {
      const size_t kc = std::find(C.inst.begin(), C.inst.end(), pr.id) - C.inst.begin();
      pr.off2 = C.off[kc];
    }
  }
  for (int l = 0; l < maxlev; ++l) {
    BLevel<T>& V = mg.L[l];
    if (V.smooth.n()) {
      V.smooth.oblocks = op_batch_plan<T>(V.smooth.h.data(), V.smooth.n(), kchunk);
      V.smooth.vblocks = vec_batch_plan(V.smooth.h.data(), V.smooth.n(), 1, kBatchVecBlocks);
      V.prolong.vblocks = vec_batch_plan(V.prolong.h.data(), V.prolong.n(), 1, kBatchVecBlocks);
    }
    if (V.restr.n()) V.restr.vblocks = vec_batch_plan(V.restr.h.data(), V.restr.n(), 1, kBatchVecBlocks);
    const std::string s = std::string(sizeof(T) == 8 ? "btab64_" : "btab32_") + std::to_string(l);
    if (!upload(c, V.smooth, s + "s") || !upload(c, V.coarse, s + "c") || !upload(c, V.restr, s + "r") ||
        !upload(c, V.prolong, s + "p"))
      return false;
    for (const BatchInst& b : V.coarse.h) {
      launch_diag<T>(b.g, b.m, V.fac + b.eoff, mg.K, mg.quirk, (T)b.sigma, nullptr, V.dinv + b.off, c.st);
      c.launches++;
    }
  }
  mg.idx32 = true;
  for (const Grid& g : g0) mg.idx32 = mg.idx32 && g.ndof() < (1LL << 30) && g.nelem() < (1LL << 30);
  return true;
}

// Copies n values from host or device memory (cudaMemcpyDefault, UVA).
bool copy_in(Ctx& c, void* dst, const void* src, size_t bytes) {
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c.st) == cudaSuccess;
}

template <typename T>
BatchInst base_inst(const Grid& g, uint32_t faces, long long off, long long noff, long long eoff, int id) {
  BatchInst b;
  std::memset(&b, 0, sizeof(b));
  b.g = g;
  b.m.faces = faces;
  b.off = off;
  b.noff = noff;
  b.eoff = eoff;
  b.id = id;
  return b;
}

}  // namespace

int batch_problem(Ctx& c, int count, const hexa_grid* grids, const hexa_bc* bcs, double nu,
                  const double* const* factors, const double* const* forces, const hexa_solve_params& prm,
                  double* const* u_out, hexa_solve_stats* stats) {
  using T = float;
  if (prm.precond != HEXA_PRECOND_MULTIGRID) {
    c.err = "batched solves use the multigrid preconditioner";
    return HEXA_ERR_ARG;
  }
  if (prm.precision == HEXA_PREC_FP64) {
    c.err = "batched solves run in mixed precision (FP32 GMG-PCG with FP64 reliable updates)";
    return HEXA_ERR_ARG;
  }
  for (int i = 0; i < count; ++i) {
    if (grids[i].dx != grids[0].dx || grids[i].dy != grids[0].dy || grids[i].dz != grids[0].dz) {
      c.err = "every instance of a batch must have the same element size";
      return HEXA_ERR_ARG;
    }
    if (bcs && bcs[i].fixed_dof) {
      c.err = "batched solves take clamp-face boundary conditions only (fixed_dof must be NULL)";
      return HEXA_ERR_ARG;
    }
  }
  cudaEventRecord(c.ev[0], c.st);
  ModalK<double> K64;
  std::string e;
  if (!build_modal(grids[0].dx, grids[0].dy, grids[0].dz, nu, &K64, &e)) {
    c.err = e;
    return HEXA_ERR_ARG;
  }
  std::vector<Grid> g0(count);
  std::vector<uint32_t> faces(count);
  std::vector<long long> off(count), eoff(count);
  long long ndof = 0, nelem = 0;
  for (int i = 0; i < count; ++i) {
    g0[i] = make_grid(grids[i].nx, grids[i].ny, grids[i].nz);
    faces[i] = bcs ? bcs[i].clamp_faces : 0u;
    off[i] = ndof;
    eoff[i] = nelem;
    ndof += g0[i].ndof();
    nelem += g0[i].nelem();
  }
  double* fac64 = c.vec<double>("bat_fac64", nelem);
  double* f64 = c.vec<double>("bat_f64", ndof);
  double* u64 = c.vec<double>("bat_u64", ndof);
  double* r64 = c.vec<double>("bat_r64", ndof);
  double* small = c.vec<double>("bat_small", 8 * (size_t)count + 64);
  T* fac32 = c.vec<T>("bat_fac32", nelem);
  T* x = c.vec<T>("bat_x", ndof);
  T* r = c.vec<T>("bat_r", ndof);
  T* zA = c.vec<T>("bat_zA", ndof);
  T* zB = c.vec<T>("bat_zB", ndof);
  T* p = c.vec<T>("bat_p", ndof);
  T* q = c.vec<T>("bat_q", ndof);
  BatchCtx B{c, count, c.vec<PcgScalars>("bat_scalars", count), c.vec<unsigned>("bat_ticket", count)};
  if (!fac64 || !f64 || !u64 || !r64 || !small || !fac32 || !x || !r || !zA || !zB || !p || !q || !B.s || !B.ticket)
    return HEXA_ERR_NOMEM;
  double *rn2 = small, *fn2 = small + count, *scale = small + 2 * count, *coef = small + 3 * count,
         *mx = small + 4 * count, *comp = small + 5 * count;
  cudaMemsetAsync(B.ticket, 0, sizeof(unsigned) * count, c.st);
  std::vector<BatchInst> base(count);
  for (int i = 0; i < count; ++i) {
    base[i] = base_inst<T>(g0[i], faces[i], off[i], off[i] / 3, eoff[i], i);
    if (!copy_in(c, fac64 + eoff[i], factors[i], sizeof(double) * g0[i].nelem()) ||
        !copy_in(c, r64 + off[i], forces[i], sizeof(double) * g0[i].ndof())) {
      cudaGetLastError();
      c.err = "batch input copy failed (instance " + std::to_string(i) + ")";
      return HEXA_ERR_ARG;
    }
    launch_mask_copy<double, double>(g0[i], base[i].m, f64 + off[i], r64 + off[i], c.st);  // loads at fixed DOFs dropped
    c.launches++;
  }
  launch_convert<float, double>(fac32, fac64, nelem, c.st);
  launch_fill<double>(u64, 0.0, ndof, c.st);
  launch_fill<T>(p, T(0), ndof, c.st);
  c.launches += 3;
  if (!c.ensure_partials((size_t)4 * kBatchVecBlocks + 4096)) return HEXA_ERR_NOMEM;
  // sigma_i = shift_factor * max diag of instance i (diagonal into r64 as scratch)
  for (int i = 0; i < count; ++i) {
    launch_diag<double>(g0[i], base[i].m, fac64 + eoff[i], K64, prm.diag_quirk, 0.0, r64 + off[i], nullptr, c.st);
    RedArgs rm;
    rm.partials = c.partials;
    rm.ticket = c.ticket;
    rm.dst = mx + i;
    rm.s = nullptr;
    rm.op = FIN_STORE;
    rm.nsum = 1;
    // about 1024 values per block: the last block's fold over the block
    // maxima is serial, so small instances get few blocks
    const int mb = (int)std::min<long long>(152 * 4, std::max<long long>(1, (g0[i].ndof() + 1023) / 1024));
    launch_max(r64 + off[i], g0[i].ndof(), rm, mb, c.st);
    c.launches += 2;
  }
  DevTable fine64;
  fine64.h = base;
  fine64.vblocks = vec_batch_plan(fine64.h.data(), count, 0, kBatchVecBlocks);
  std::vector<double> hmax(count), hf(count), sigma(count);
  cudaMemcpyAsync(hmax.data(), mx, sizeof(double) * count, cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("batch setup")) return HEXA_ERR_CUDA;
  for (int i = 0; i < count; ++i) {
    if (std::isnan(hmax[i]) || std::isinf(hmax[i])) {
      c.err = "Stiffness Matrix Diagonal contains NaN/Inf (instance " + std::to_string(i) + ")";
      return HEXA_ERR_CORRUPT_INPUT;
    }
    sigma[i] = prm.shift_factor * hmax[i];
    fine64.h[i].sigma = sigma[i];
    base[i].sigma = sigma[i];
  }
  fine64.oblocks = op_batch_plan<double>(fine64.h.data(), count, 0);
  if (!upload(c, fine64, "bat_tab64")) return HEXA_ERR_NOMEM;
  launch_batch_dot<double>(fine64.d, count, fine64.vblocks, 0, f64, f64, nullptr, nullptr, bred(B, FIN_STORE, 1, fn2),
                           nullptr, c.st);
  c.launches++;
  cudaMemcpyAsync(hf.data(), fn2, sizeof(double) * count, cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("batch setup")) return HEXA_ERR_CUDA;
  std::vector<double> fnorm(count);
  for (int i = 0; i < count; ++i) fnorm[i] = std::sqrt(std::max(hf[i], 0.0));

  // hierarchy and smoother
  BatchMG<T> mg;
  mg.K = modal_to_f32(K64);
  mg.quirk = prm.diag_quirk;
  {
    double ke[576];
    canonical_stiffness(grids[0].dx, grids[0].dy, grids[0].dz, nu, ke);
    const double lmax = smoother_bound(ke, prm.diag_quirk);
    mg.cheb = prm.smoother == HEXA_SMOOTH_CHEBYSHEV;
    mg.omega = (T)(prm.jacobi_omega > 0 ? prm.jacobi_omega : 1.2 / lmax);
    mg.nu1 = prm.pre_smooth > 0 ? prm.pre_smooth : 1;
    mg.nu2 = prm.post_smooth >= 0 ? prm.post_smooth : 2;
    mg.citers = prm.coarse_iters >= 0 ? prm.coarse_iters : 30;
    const int nmax = std::max(mg.nu1, mg.nu2) + 1;
    const double lmin = lmax / (prm.cheb_ratio > 1 ? prm.cheb_ratio : 10.0), th = 0.5 * (lmax + lmin), de = 0.5 * (lmax - lmin), sg = th / de;
    double rho = 1.0 / sg;
    mg.inv_theta = (T)(1.0 / th);
    mg.c1.assign(nmax + 1, T(0));
    mg.c2.assign(nmax + 1, T(0));
    for (int s = 1; s <= nmax; ++s) {
      const double rn = 1.0 / (2.0 * sg - rho);
      mg.c1[s] = (T)(rn * rho);
      mg.c2[s] = (T)(2.0 * rn / de);
      rho = rn;
    }
  }
  std::vector<int> nlev(count);
  for (int i = 0; i < count; ++i) nlev[i] = batch_levels(g0[i], faces[i], prm.mg_levels);
  int kchunk = 16;
  const std::string tkey = "batch/" + std::to_string(count) + "/" + std::to_string(nelem) + "/" + std::to_string(ndof);
  bool tuned = false;
  if (prm.autotune) {
    auto it = c.tuned.find(tkey);
    if (it != c.tuned.end()) kchunk = it->second.a, tuned = true;
  }
  if (!build_batch_mg<T>(c, mg, g0, faces, sigma, nlev, fac32, kchunk)) return HEXA_ERR_NOMEM;
  if (prm.autotune && !tuned && mg.L[0].smooth.n()) {
    // z-brick depth: time the fine-level batched Chebyshev sweep for 8, 16 and 32 layers
    launch_fill<T>(zA, T(0), ndof, c.st);
    launch_fill<T>(r, T(0), ndof, c.st);
    c.launches += 2;
    double best = INFINITY;
    int bestk = 16;
    for (int kc : {8, 16, 32}) {
      DevTable t;
      t.h = mg.L[0].smooth.h;
      t.oblocks = op_batch_plan<T>(t.h.data(), t.n(), kc);
      if (!upload(c, t, "bat_tune")) return HEXA_ERR_NOMEM;
      BatchOpArgs<T> a = bop<T>(B, mg.K, mg.quirk, t, fac32, zA, r, zB, nullptr, mg.c1[1], mg.c2[1], T(0),
                                bred(B, FIN_NONE, 1));
      a.s = nullptr;
      launch_op_batch<T>(OP_CHEB2, a, mg.idx32, c.st);
      cudaEventRecord(c.ev[2], c.st);
      for (int rep = 0; rep < 5; ++rep) launch_op_batch<T>(OP_CHEB2, a, mg.idx32, c.st);
      cudaEventRecord(c.ev[3], c.st);
      if (cudaEventSynchronize(c.ev[3]) != cudaSuccess) return c.cuda_ok("batch tune") ? HEXA_ERR_CUDA : HEXA_ERR_CUDA;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c.ev[2], c.ev[3]);
      c.launches += 6;
      if (ms < best) best = ms, bestk = kc;
    }
    c.tuned[tkey] = {bestk, 0, 0};
    kchunk = bestk;
    if (!build_batch_mg<T>(c, mg, g0, faces, sigma, nlev, fac32, kchunk)) return HEXA_ERR_NOMEM;
  }
  DevTable fine;
  fine.h = base;
  fine.oblocks = op_batch_plan<T>(fine.h.data(), count, kchunk);
  fine.vblocks = vec_batch_plan(fine.h.data(), count, 0, kBatchVecBlocks);
  if (!upload(c, fine, "bat_tab32")) return HEXA_ERR_NOMEM;
  const int maxb = std::max({fine.oblocks, fine.vblocks, fine64.oblocks, fine64.vblocks, 4 * kBatchVecBlocks});
  if (!c.ensure_partials((size_t)maxb * 2 + 4096)) return HEXA_ERR_NOMEM;
  if (!c.cuda_ok("batch setup")) return HEXA_ERR_CUDA;
  cudaEventRecord(c.ev[1], c.st);

  const int G0 = prm.graph_iters > 0 ? prm.graph_iters : 10;
  const int G = (G0 & 1) ? G0 + 1 : G0;  // even: each group starts on the same z buffer
  auto iteration = [&](int parity) {
    T* zc = parity == 0 ? zB : zA;
    T* zo = parity == 0 ? zA : zB;
    launch_op_batch<T>(OP_APPLY_DOT, bop<T>(B, mg.K, mg.quirk, fine, fac32, p, nullptr, q, nullptr, T(0), T(0), T(0),
                                            bred(B, FIN_PCG_ALPHA, 1)),
                       mg.idx32, c.st);
    launch_batch_pcg_update<T>(fine.d, count, fine.vblocks, 0, x, r, nullptr, p, q, nullptr, bred(B, FIN_PCG_RES, 1),
                               B.s, c.st);
    c.launches += 2;
    bvcycle<T>(B, mg, 0, r, zc);
    launch_batch_dot<T>(fine.d, count, fine.vblocks, 0, r, zc, r, zo, bred(B, FIN_PCG_BETA, 2), B.s, c.st);
    launch_batch_p_update<T>(fine.d, count, fine.vblocks, 0, p, zc, B.s, c.st);
    c.launches += 2;
  };
  BatchOpArgs<double> ares;
  ares.K = K64;
  ares.c1 = ares.c2 = ares.omega = 0.0;
  ares.diag_quirk = prm.diag_quirk;
  ares.inst = fine64.d;
  ares.ninst = count;
  ares.nblocks = fine64.oblocks;
  ares.x = u64;
  ares.fac = fac64;
  ares.b = f64;
  ares.y = r64;
  ares.xin = nullptr;
  ares.red = bred(B, FIN_STORE, 1, rn2);
  ares.s = nullptr;

  std::vector<PcgScalars> hs(count);
  for (auto& h : hs) {
    std::memset(&h, 0, sizeof(h));
    h.bnorm = 1.0;
    h.best_rel = INFINITY;
    h.max_iter = prm.max_iter;
    h.cadence = prm.check_cadence;
    h.no_div = 1;
  }
  std::vector<double> rel(count, 0.0), sc_old(count, 0.0), rz_old(count, 0.0), hn(count);
  const double inner_tol = prm.inner_tol > 0 ? prm.inner_tol : 1e-4;
  const int max_outer = prm.max_outer > 0 ? prm.max_outer : 20;
  int outer = 0, status = HEXA_OK, applies64 = 0;
  cudaGraphExec_t gexec = nullptr;
  int64_t gnodes = 0;
  auto fail = [&](const char* where) {
    if (gexec) cudaGraphExecDestroy(gexec);
    c.cuda_ok(where);
    return HEXA_ERR_CUDA;
  };
  while (true) {
    launch_op_batch<double>(OP_RESID_NORM, ares, mg.idx32, c.st);  // FP64 true residuals
    c.launches++;
    ++applies64;
    cudaMemcpyAsync(hn.data(), rn2, sizeof(double) * count, cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess) return fail("batch residual");
    bool done = true, bad = false, exhausted = outer >= max_outer;
    for (int i = 0; i < count; ++i) {
      rel[i] = fnorm[i] > 0 ? std::sqrt(std::max(hn[i], 0.0)) / fnorm[i] : 0.0;
      if (!(rel[i] == rel[i])) bad = true;
      if (rel[i] > prm.tol) {
        done = false;
        if (hs[i].iter >= prm.max_iter || hs[i].status == 2) exhausted = true;
      }
    }
    if (done) break;
    if (bad || exhausted) {
      status = HEXA_NOT_CONVERGED;
      break;
    }
    // active instances restart from their unit-norm FP64 residual; the search
    // direction is kept: p <- z + rz_new / (rz_old * ratio) p
    std::vector<double> hscale(count), hcoef(count);
    for (int i = 0; i < count; ++i) {
      const double rn = rel[i] * fnorm[i];
      const bool active = rel[i] > prm.tol && rn > 0.0;
      hscale[i] = active ? 1.0 / rn : 0.0;
      const double ratio = sc_old[i] > 0 ? hscale[i] / sc_old[i] : 0.0;
      hcoef[i] = (active && ratio > 0 && rz_old[i] > 0) ? 1.0 / (rz_old[i] * ratio) : 0.0;
      PcgScalars& h = hs[i];
      h.halt = active ? 0 : 1;
      h.status = 0;
      h.tol = std::max(inner_tol, 0.5 * prm.tol / std::max(rel[i], 1e-300));
      h.best_rel = INFINITY;
      h.bnorm = 1.0;
    }
    cudaMemcpyAsync(scale, hscale.data(), sizeof(double) * count, cudaMemcpyHostToDevice, c.st);
    cudaMemcpyAsync(coef, hcoef.data(), sizeof(double) * count, cudaMemcpyHostToDevice, c.st);
    cudaMemcpyAsync(B.s, hs.data(), sizeof(PcgScalars) * count, cudaMemcpyHostToDevice, c.st);
    launch_batch_from64<T>(fine.d, count, fine.vblocks, r, r64, scale, c.st);
    launch_fill<T>(x, T(0), ndof, c.st);
    c.launches += 2;
    bvcycle<T>(B, mg, 0, r, zA);
    launch_batch_dot<T>(fine.d, count, fine.vblocks, 0, r, zA, nullptr, nullptr, bred(B, FIN_INIT_RZ, 1), B.s, c.st);
    launch_batch_set_beta(B.s, coef, count, c.st);
    launch_batch_p_update<T>(fine.d, count, fine.vblocks, 0, p, zA, B.s, c.st);
    c.launches += 3;
    if (prm.use_graphs && !gexec) {
      cudaGraph_t gr = nullptr;
      if (cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fail("batch capture");
      const int64_t before = c.launches;
      for (int it = 0; it < G; ++it) iteration(it & 1);
      gnodes = c.launches - before;
      c.launches = before;
      const cudaError_t e1 = cudaStreamEndCapture(c.st, &gr);
      const cudaError_t e2 = e1 == cudaSuccess ? cudaGraphInstantiate(&gexec, gr, 0) : e1;
      if (gr) cudaGraphDestroy(gr);
      if (e2 != cudaSuccess) {
        gexec = nullptr;
        return fail("batch graph");
      }
    }
    // bounded by the per-instance iteration caps: every group advances each active instance
    const long long max_groups = (long long)prm.max_iter / G + 2;
    for (long long grp = 0; grp < max_groups; ++grp) {
      if (prm.use_graphs) {
        if (cudaGraphLaunch(gexec, c.st) != cudaSuccess) return fail("batch graph launch");
        c.launches += gnodes;
      } else {
        for (int it = 0; it < G; ++it) iteration(it & 1);
      }
      cudaMemcpyAsync(hs.data(), B.s, sizeof(PcgScalars) * count, cudaMemcpyDeviceToHost, c.st);
      if (cudaStreamSynchronize(c.st) != cudaSuccess) return fail("batch pcg");
      bool all = true;
      for (const PcgScalars& h : hs) all = all && h.halt;
      if (all) break;
    }
    ++outer;
    for (int i = 0; i < count; ++i) {
      sc_old[i] = hscale[i];
      rz_old[i] = hs[i].rz;
    }
    launch_batch_accum<T>(fine.d, count, fine.vblocks, u64, x, scale, c.st);
    c.launches++;
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  launch_batch_dot<double>(fine64.d, count, fine64.vblocks, 0, f64, u64, nullptr, nullptr, bred(B, FIN_STORE, 1, comp),
                           nullptr, c.st);
  c.launches++;
  for (int i = 0; i < count; ++i)
    cudaMemcpyAsync(u_out[i], u64 + off[i], sizeof(double) * g0[i].ndof(), cudaMemcpyDefault, c.st);
  std::vector<double> hcomp(count);
  cudaMemcpyAsync(hcomp.data(), comp, sizeof(double) * count, cudaMemcpyDeviceToHost, c.st);
  cudaEventRecord(c.ev[2], c.st);
  if (cudaEventSynchronize(c.ev[2]) != cudaSuccess || !c.cuda_ok("batch solve")) return HEXA_ERR_CUDA;
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, c.ev[0], c.ev[1]);
  cudaEventElapsedTime(&ms2, c.ev[1], c.ev[2]);
  c.last_ms = ms1 + ms2;
  if (stats) {
    for (int i = 0; i < count; ++i) {
      hexa_solve_stats& st = stats[i];
      std::memset(&st, 0, sizeof(st));
      st.status = rel[i] <= prm.tol ? HEXA_OK : HEXA_NOT_CONVERGED;
      st.iterations = hs[i].iter;
      st.outer_iterations = outer;
      st.attempts = 1;
      st.precond_used = HEXA_PRECOND_USED_MULTIGRID;
      st.mg_levels = nlev[i];
      st.smooth_steps = mg.nu2;
      st.relres = rel[i];
      st.true_relres = rel[i];
      st.unshifted_relres = sigma[i] == 0.0 ? rel[i] : NAN;  // not recomputed for shifted batches
      st.shift = sigma[i];
      st.max_diag = hmax[i];
      st.compliance = hcomp[i];
      st.setup_ms = ms1;
      st.solve_ms = ms2;
      st.fine_applies_fp64 = applies64;
    }
  }
  return status;
}

// ---------------------------------------------------------------- filter
template <typename T>
int batch_filter_t(Ctx& c, int count, const hexa_grid* grids, const double* const* rho_in, const HelmK& K, double tol,
                   int max_iter, double* const* rho_out, hexa_filter_stats* stats) {
  std::vector<Grid> g(count);
  std::vector<long long> noff(count), eoff(count);
  long long nn = 0, ne = 0;
  for (int i = 0; i < count; ++i) {
    g[i] = make_grid(grids[i].nx, grids[i].ny, grids[i].nz);
    noff[i] = nn;
    eoff[i] = ne;
    nn += g[i].nnode();
    ne += g[i].nelem();
  }
  const char* tg = sizeof(T) == 8 ? "bh64_" : "bh32_";
  auto nm = [&](const char* s) { return std::string(tg) + s; };
  double* rho64 = c.vec<double>(nm("rho64"), ne);
  T* rho = c.vec<T>(nm("rho"), ne);
  T* b = c.vec<T>(nm("b"), nn);
  T* x = c.vec<T>(nm("x"), nn);
  T* r = c.vec<T>(nm("r"), nn);
  T* z = c.vec<T>(nm("z"), nn);
  T* p = c.vec<T>(nm("p"), nn);
  T* q = c.vec<T>(nm("q"), nn);
  T* dinv = c.vec<T>(nm("dinv"), nn);
  T* outT = c.vec<T>(nm("out"), ne);
  double* out64 = c.vec<double>(nm("out64"), ne);
  double* small = c.vec<double>(nm("small"), 2 * (size_t)count + 8);
  BatchCtx B{c, count, c.vec<PcgScalars>(nm("scalars"), count), c.vec<unsigned>(nm("ticket"), count)};
  if (!rho64 || !rho || !b || !x || !r || !z || !p || !q || !dinv || !outT || !out64 || !small || !B.s || !B.ticket)
    return HEXA_ERR_NOMEM;
  cudaMemsetAsync(B.ticket, 0, sizeof(unsigned) * count, c.st);
  DevTable t;
  for (int i = 0; i < count; ++i) {
    t.h.push_back(base_inst<T>(g[i], 0u, 3 * noff[i], noff[i], eoff[i], i));
    if (!copy_in(c, rho64 + eoff[i], rho_in[i], sizeof(double) * g[i].nelem())) {
      cudaGetLastError();
      c.err = "batch filter input copy failed (instance " + std::to_string(i) + ")";
      return HEXA_ERR_ARG;
    }
  }
  t.vblocks = vec_batch_plan(t.h.data(), count, 1, kBatchVecBlocks);
  if (!upload(c, t, nm("tab")) || !c.ensure_partials((size_t)t.vblocks * 2 + 4096)) return HEXA_ERR_NOMEM;
  if constexpr (sizeof(T) == 8) cudaMemcpyAsync(rho, rho64, sizeof(double) * ne, cudaMemcpyDeviceToDevice, c.st);
  else launch_convert<float, double>(rho, rho64, ne, c.st);
  for (int i = 0; i < count; ++i) {
    launch_helm_rhs<T>(g[i], rho + eoff[i], (T)K.rhs_scale, b + noff[i], c.st);
    launch_helm_dinv<T>(g[i], K, dinv + noff[i], c.st);
  }
  c.launches += 1 + 2 * count;
  launch_batch_dot<T>(t.d, count, t.vblocks, 1, b, b, nullptr, nullptr, bred(B, FIN_STORE, 1, small), nullptr, c.st);
  c.launches++;
  std::vector<double> bb(count);
  cudaMemcpyAsync(bb.data(), small, sizeof(double) * count, cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("batch filter setup")) return HEXA_ERR_CUDA;
  std::vector<PcgScalars> hs(count);
  for (int i = 0; i < count; ++i) {
    PcgScalars& h = hs[i];
    std::memset(&h, 0, sizeof(h));
    h.tol = tol;
    h.max_iter = max_iter;
    h.cadence = -10;  // GPUHelmholtz.jl:245: test every 10 iterations
    h.no_div = 1;
    h.bnorm = std::sqrt(std::max(bb[i], 0.0));
    h.best_rel = INFINITY;
    h.halt = h.bnorm == 0.0 ? 1 : 0;  // GPUHelmholtz.jl:203-206: zero input comes back unchanged
  }
  cudaMemcpyAsync(B.s, hs.data(), sizeof(PcgScalars) * count, cudaMemcpyHostToDevice, c.st);
  launch_fill<T>(x, T(0), nn, c.st);
  launch_copy<T>(r, b, nn, c.st);
  launch_cols_jacobi<T>(z, r, dinv, nn, 1, nullptr, c.st);
  launch_batch_dot<T>(t.d, count, t.vblocks, 1, r, z, nullptr, nullptr, bred(B, FIN_INIT_RZ, 1), B.s, c.st);
  launch_copy<T>(p, z, nn, c.st);
  c.launches += 5;
  auto iteration = [&]() {
    launch_batch_helm_apply_dot<T>(t.d, count, t.vblocks, K, p, q, bred(B, FIN_PCG_ALPHA, 1), B.s, c.st);
    launch_batch_pcg_update<T>(t.d, count, t.vblocks, 1, x, r, z, p, q, dinv, bred(B, FIN_PCG_RES, 2), B.s, c.st);
    launch_batch_p_update<T>(t.d, count, t.vblocks, 1, p, z, B.s, c.st);
    c.launches += 3;
  };
  const long long max_groups = (long long)max_iter / 10 + 2;
  for (long long grp = 0; grp < max_groups; ++grp) {
    for (int it = 0; it < 10; ++it) iteration();
    cudaMemcpyAsync(hs.data(), B.s, sizeof(PcgScalars) * count, cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("batch filter")) return HEXA_ERR_CUDA;
    bool all = true;
    for (const PcgScalars& h : hs) all = all && h.halt;
    if (all) break;
  }
  for (int i = 0; i < count; ++i) {
    if (hs[i].bnorm == 0.0) {
      cudaMemcpyAsync(out64 + eoff[i], rho64 + eoff[i], sizeof(double) * g[i].nelem(), cudaMemcpyDeviceToDevice, c.st);
      continue;
    }
    launch_helm_extract<T>(g[i], x + noff[i], outT + eoff[i], c.st);
    c.launches++;
    if constexpr (sizeof(T) == 8) {
      cudaMemcpyAsync(out64 + eoff[i], outT + eoff[i], sizeof(double) * g[i].nelem(), cudaMemcpyDeviceToDevice, c.st);
    } else {
      launch_convert<double, float>(out64 + eoff[i], outT + eoff[i], g[i].nelem(), c.st);
      c.launches++;
    }
  }
  for (int i = 0; i < count; ++i)
    cudaMemcpyAsync(rho_out[i], out64 + eoff[i], sizeof(double) * g[i].nelem(), cudaMemcpyDefault, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("batch filter")) return HEXA_ERR_CUDA;
  if (stats)
    for (int i = 0; i < count; ++i) {
      std::memset(&stats[i], 0, sizeof(hexa_filter_stats));
      stats[i].status = HEXA_OK;
      stats[i].iterations = hs[i].iter;
      stats[i].relres = hs[i].relres;
    }
  return HEXA_OK;
}

int batch_filter(Ctx& c, int count, const hexa_grid* grids, const double* const* rho_in, double radius, double tol,
                 int max_iter, int quirk, int precision, double* const* rho_out, hexa_filter_stats* stats) {
  for (int i = 0; i < count; ++i)
    if (grids[i].dx != grids[0].dx || grids[i].dy != grids[0].dy || grids[i].dz != grids[0].dz) {
      c.err = "every instance of a batch must have the same element size";
      return HEXA_ERR_ARG;
    }
  double Ke[64], Me[64];
  if (scalar_matrices(grids[0].dx, grids[0].dy, grids[0].dz, quirk, Ke, Me) != 0) {
    c.err = "invalid element size";
    return HEXA_ERR_ARG;
  }
  HelmK K;
  helm_corner_matrix(Ke, Me, radius, K.A);
  K.rhs_scale = grids[0].dx * grids[0].dy * grids[0].dz / 8.0;
  return precision == HEXA_PREC_FP32 ? batch_filter_t<float>(c, count, grids, rho_in, K, tol, max_iter, rho_out, stats)
                                     : batch_filter_t<double>(c, count, grids, rho_in, K, tol, max_iter, rho_out, stats);
}

}  // namespace hexa
