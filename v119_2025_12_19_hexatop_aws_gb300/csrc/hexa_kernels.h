// Launch-side declarations of every kernel of the hex8 solve path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hexa_common.cuh"

namespace hexa {

// ---------------------------------------------------------------- operator
enum OpMode {
  OP_APPLY = 0,       // y = Ax
  OP_APPLY_DOT = 1,   // y = Ax, sum x.Ax
  OP_RESID = 2,       // y = b - Ax
  OP_RESID_NORM = 3,  // y = b - Ax, sum y.y
  OP_JACOBI = 4,      // y = x + omega D^-1 (b - Ax)
  OP_CHEB2 = 5,       // y = x + c1 (x - xin) + c2 D^-1 (b - Ax)   (xin null: 0; y may alias xin)
  OP_JACOBI_DOT = 6,  // OP_JACOBI, sum b.y (r.z of the V-cycle's last step)
  OP_CHEB2_DOT = 7,   // OP_CHEB2, sum b.y
};

template <typename T>
struct OpArgs {
  Grid g;
  Mask m;
  const T* x;     // stencil input, zero at fixed DOFs
  const T* fac;   // element factors (nelem)
  const T* b;     // right-hand side (RESID*, JACOBI)
  T* y;           // output (must not alias x)
  const T* xin;   // Chebyshev: previous iterate (nullable = 0)
  T c1, c2;       // Chebyshev step coefficients
  ModalK<T> K;
  T sigma;        // diagonal shift
  T omega;        // Jacobi damping
  int kchunk;     // node layers per work item
  int tiles_x, tiles_y, nchunks;  // filled by launch_op
  int diag_quirk;
  RedArgs red;
  const int* halt;  // nullable: PcgScalars::halt
  int ncol = 1;     // columns (x, b, xin, y advance by ndof per column): OP_APPLY,
                    // OP_RESID, OP_JACOBI and OP_CHEB2 only
  int test_stall = -1;  // FP32 staged form: layer load that CTA 0 leaves out (tests of the bounded waits)
};

template <typename T>
void launch_op(int mode, const OpArgs<T>& a, cudaStream_t st);
// Whether a staged FP32 operator launch gave up a bounded wait since the last
// call (reads and clears the device word; synchronizes st).
bool op_take_wait_error(cudaStream_t st);
template <typename T>
long long op_num_blocks(const Grid& g, int kchunk);
// node layers per work item so that every resident CTA gets ~8 items
template <typename T>
int op_pick_kchunk(const Grid& g);
ModalK<float> modal_to_f32(const ModalK<double>& K);

// ------------------------------------------------------------ vector passes
// All vectors are full-length AoS (3*nNodes) and zero at fixed DOFs.  The
// PCG passes take n = the length of one column; with RedArgs::ncol > 1 they
// work on ncol consecutive columns (per-column scalars and reductions; a
// diagonal is shared by the columns).
template <typename T>
void launch_fill(T* v, T val, long long n, cudaStream_t st);
template <typename T>
void launch_copy(T* dst, const T* src, long long n, cudaStream_t st);
// dst = src with fixed DOFs zeroed (expand/contract semantics)
template <typename TD, typename TS>
void launch_mask_copy(const Grid& g, const Mask& m, TD* dst, const TS* src, cudaStream_t st);
// Jacobi inverse diagonal dinv = 1/(dd*fsum + sigma) (0 at fixed DOFs) and
// the raw diagonal (dd*fsum, 0 at fixed DOFs).
template <typename T>
void launch_diag(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, int quirk, T sigma,
                 T* diag, T* dinv, cudaStream_t st);
// max over the vector (non-negative entries), result into *dst (device)
void launch_max(const double* v, long long n, const RedArgs& red, int nblocks, cudaStream_t st);
// sums: dst = [a.b]  or [a.b, c.d]
template <typename T>
void launch_dot(const T* a, const T* b, const T* c, const T* d, long long n, const RedArgs& red,
                int nblocks, const int* halt, cudaStream_t st);
// PCG update: x += alpha p; r -= alpha q; rr = r.r ; with dinv: z = dinv*r, rz = r.z
template <typename T>
void launch_pcg_update(T* x, T* r, T* z, const T* p, const T* q, const T* dinv, long long n,
                       const RedArgs& red, int nblocks, const PcgScalars* s, cudaStream_t st);
// p = z + beta p
template <typename T>
void launch_p_update(T* p, const T* z, long long n, const PcgScalars* s, cudaStream_t st, int ncol = 1);
// x += alpha p, r -= alpha q; sums ||r||^2 and r.zo (FIN_PCG_RES_MG), one column
template <typename T>
void launch_pcg_update_mg(T* x, T* r, const T* p, const T* q, const T* zo, long long n, const RedArgs& red,
                          int nblocks, const PcgScalars* s, cudaStream_t st);

// z = dinv * r (Jacobi) ; rz = r.z
template <typename T>
void launch_jacobi_precond(T* z, const T* r, const T* dinv, long long n, const RedArgs& red,
                           int nblocks, const int* halt, cudaStream_t st);
// dst32 = (T32)(src64 * scale)
void launch_scale_to_f32(float* dst, const double* src, const double* scale, long long n,
                         cudaStream_t st, int ncol = 1);
// u64 += (double)d32 / scale
void launch_add_scaled_f32(double* u, const float* d, const double* scale, long long n,
                           cudaStream_t st, int ncol = 1);
// x = a*x + b*y with host scalars
template <typename T>
void launch_axpby(T* x, T a, const T* y, T b, long long n, cudaStream_t st);

// ---------------------------------------------------------------- multigrid
// coarse factor = 2 * mean of the 8 children (rediscretised K0 at 2h = 2*K0(h))
template <typename T>
void launch_coarsen_factors(const Grid& gf, const T* ff, const Grid& gc, T* fc, cudaStream_t st);
template <typename TD, typename TS>
void launch_convert(TD* dst, const TS* src, long long n, cudaStream_t st);
// coarse node mask by injection
void launch_coarsen_mask(const Grid& gf, const uint8_t* mf, const Grid& gc, uint8_t* mc,
                         cudaStream_t st);
// b_c = P^T r_f (full weighting, 27 fine nodes per coarse node).  This and
// the two passes below take ncol columns (vectors ndof of their grid apart)
// and return the number of launches issued.
template <typename T>
int launch_restrict(const Grid& gf, const T* rf, const Grid& gc, const Mask& mc, T* bc,
                    const int* halt, cudaStream_t st, int ncol = 1);
// x_f += P x_c (trilinear)
template <typename T>
int launch_prolong_add(const Grid& gc, const T* xc, const Grid& gf, const Mask& mf, T* xf,
                       const int* halt, cudaStream_t st, int ncol = 1);
// `iters` Jacobi-PCG iterations on a small grid in one single-CTA launch
// (w: 24 * nelem scratch for the element products)
template <typename T>
void launch_coarse_pcg(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, T sigma, const T* dinv,
                       const T* b, T* x, T* r, T* z, T* p, T* q, T* w, int iters, const int* halt, cudaStream_t st);
// x = omega * b / D (first damped-Jacobi sweep from a zero guess)
template <typename T>
int launch_jacobi0(const Grid& g, const Mask& m, const T* fac, const ModalK<T>& K, int quirk,
                   T sigma, T omega, const T* b, T* x, const int* halt, cudaStream_t st, int ncol = 1);

// --------------------------------------------------------------- Helmholtz
struct HelmK {
  double A[8][8];  // R^2 Ke + Me, corner order dx + 2dy + 4dz
  double rhs_scale; // vol/8
};
template <typename T>
void launch_helm_rhs(const Grid& g, const T* rho, T scale, T* b, cudaStream_t st);
template <typename T>
void launch_helm_apply_dot(const Grid& g, const HelmK& K, const T* x, T* y, const RedArgs& red,
                           int nblocks, const int* halt, cudaStream_t st);
template <typename T>
void launch_helm_dinv(const Grid& g, const HelmK& K, T* dinv, cudaStream_t st);
template <typename T>
void launch_helm_extract(const Grid& g, const T* psi, T* rho_out, cudaStream_t st);

// ------------------------------------------------------------------ SIMP/OC
void launch_simp_factors(const double* rho, double Emin, double E0, double penal, double* fac,
                         long long n, cudaStream_t st);
void launch_sensitivities(const Grid& g, const ModalK<double>& K, const double* rho,
                          const double* u, double Emin, double E0, double penal, double* dc,
                          const RedArgs& red, cudaStream_t st);
void launch_oc_volumes(const double* x, const double* dc, const double* dv, long long n,
                       const double* lam, int nlam, double move, double* partials, int nblocks,
                       cudaStream_t st);
void launch_oc_apply(const double* x, const double* dc, const double* dv, long long n, double lam,
                     double move, double* xout, cudaStream_t st);


// ---- stress post-processing (stress.cu) ----------------------------------
template <typename TU>
void launch_stress(const Grid& g, const TU* u, const float* density, float E, float nu, float dx, float dy, float dz,
                   int save_voigt, float* principal, float* vonmises, float* voigt, float* l1, float* dmax,
                   float* dmin, cudaStream_t st);

// ---- density transfer onto a refined grid (remap.cu) ----------------------
void launch_remap(int onx, int ony, int onz, int nnx, int nny, int nnz, float ndx, float ndy, float ndz, float lx,
                  float ly, float lz, int projection, const float* dens, const float* alpha, float* nd, float* na,
                  cudaStream_t st);
void launch_remap_nodal(int onx, int ony, int onz, int nnx, int nny, int nnz, const double* u, double* un,
                        cudaStream_t st);

// ---- density update between solves (update.cu) -----------------------------
struct UpdateState {
  int nan_stress, nan_filtered, mode, pad;  // mode: 0 cull none, 1 every candidate, 2 the `allowed` smallest
  double change;                            // sum of |min(raw, max) - old| over unprotected elements
  unsigned long long active_updated;        // unprotected raw > min_density (the mean's divisor)
  unsigned long long active, candidates, allowed, culled;
  unsigned long long prefix, remaining;     // radix select: key of the last culled candidate
  float mean_change, pad2;
};
void launch_propose(long long n, const float* l1, const uint8_t* prot, const float* orig, float allow, float E,
                    float min_d, float* prop, UpdateState* s, cudaStream_t st);
int launch_update_cull(long long n, const float* old, const float* src, const uint8_t* prot, const float* orig,
                       float min_d, float max_d, float thr, float ratio, int hard, float* out, double* part,
                       unsigned long long* hist, UpdateState* s, cudaStream_t st);
size_t update_partials_doubles();
int update_hist_bins();

// ---- block PCG over k <= kMaxBlockCols columns (block.cu) ----------------
constexpr int kMaxBlockCols = 16;
constexpr int kBlockRedBlocks = 608;  // grid of the reducing block passes
int block_kc(int k);                  // compiled column count (1, 2, 4, 8, 16) for k
long long block_partials_needed(int k);
// out[i * NBC + j] = a_i . b_j over the columns (NBC = kc or 2 kc; b_j = b1_j,
// then b2_j when b2 is given); the last block writes out in a fixed order
template <typename T>
void launch_gram(const T* a, const T* b1, const T* b2, int k, long long n, double* partials, unsigned* ticket,
                 double* out, const int* halt, cudaStream_t st);
// out = sign * G^+ rhs (k x k, G symmetrised from g, pivots below eps * G_jj dropped)
void launch_block_solve(const double* g, int ldg, const double* r, int ldr, int roff, int k, double sign, double eps,
                        double* out, const int* halt, cudaStream_t st);
// X += P alpha, R -= Q alpha, column norms of R reduced with red (FIN_BLOCK_RES)
template <typename T>
void launch_block_update(T* X, T* R, const T* P, const T* Q, const double* alpha, int k, long long n,
                         const RedArgs& red, cudaStream_t st);
template <typename T>
void launch_block_p_update(T* P, const T* Z, const double* beta, int k, long long n, const int* halt,
                           cudaStream_t st);
template <typename T>
void launch_cols_jacobi(T* z, const T* r, const T* dinv, long long n, int k, const int* halt, cudaStream_t st);
// dst_j = (T)(src_j * scale[j])
template <typename T>
void launch_cols_from64(T* dst, const double* src, const double* scale, long long n, int k, cudaStream_t st);
// u_j += d_j / scale[j] (columns with scale 0 are left alone)
template <typename T>
void launch_cols_accum(double* u, const T* d, const double* scale, long long n, int k, cudaStream_t st);


// ---- batches of independent grids (one launch over all instances) -------
// One instance of a batched launch.  Vectors of a batch level are the
// instances' vectors back to back: DOF vectors from `off`, node vectors from
// `noff`, element arrays from `eoff`.  A launch gives instance i the blocks
// [blk0, blk0 + nblk) of its grid; reductions and halts are per instance (id).
struct BatchInst {
  Grid g;
  Mask m;
  long long off, noff, eoff;
  // the other level of a transfer (restriction: the finer grid; prolongation:
  // the coarser grid) and its DOF offset
  Grid g2;
  Mask m2;
  long long off2;
  double sigma;
  int id;
  int kchunk, tiles_x, tiles_y, nchunks;  // operator tiling
  int oblk0, onblk;                       // operator blocks
  int vblk0, vnblk;                       // vector / transfer pass blocks
  int pad;
};

// Fills the operator tiling (z-bricks of kchunk node layers, 0 = 16) and the
// block ranges of n instances (targeting the resident CTAs of the operator in
// precision T); returns the grid size.
template <typename T>
int op_batch_plan(BatchInst* in, int n, int kchunk);
// s[i].beta = s[i].rz * coef[i] for i < n (direction kept across a reliable update)
void launch_batch_set_beta(PcgScalars* s, const double* coef, int n, cudaStream_t st);
// Fills the vector-pass block ranges in proportion to units(i) (DOFs, nodes
// or elements by `unit`: 0 DOF, 1 node, 2 element, 3 node of g2); returns the grid.
int vec_batch_plan(BatchInst* in, int n, int unit, int max_blocks);

template <typename T>
struct BatchOpArgs {
  ModalK<T> K;
  T c1, c2, omega;
  int diag_quirk;
  const BatchInst* inst;  // device table
  int ninst, nblocks;
  const T* x;
  const T* fac;
  const T* b;
  T* y;
  const T* xin;
  RedArgs red;            // group = instance id
  const PcgScalars* s;    // per-instance halts (nullable)
};
template <typename T>
void launch_op_batch(int mode, const BatchOpArgs<T>& a, bool idx32, cudaStream_t st);

// vector passes over a batch (n per instance = its DOFs, or nodes if node_sized)
template <typename T>
void launch_batch_pcg_update(const BatchInst* in, int ninst, int nblocks, int node_sized, T* x, T* r, T* z,
                             const T* p, const T* q, const T* dinv, const RedArgs& red, const PcgScalars* s,
                             cudaStream_t st);
template <typename T>
void launch_batch_p_update(const BatchInst* in, int ninst, int nblocks, int node_sized, T* p, const T* z,
                           const PcgScalars* s, cudaStream_t st);
// sums a.b (and c.d when c is given) per instance
template <typename T>
void launch_batch_dot(const BatchInst* in, int ninst, int nblocks, int node_sized, const T* a, const T* b,
                      const T* c, const T* d, const RedArgs& red, const PcgScalars* s, cudaStream_t st);
// dst = (T)(src * scale[id]) ; u += d / scale[id] (scale 0: left alone)
template <typename T>
void launch_batch_from64(const BatchInst* in, int ninst, int nblocks, T* dst, const double* src,
                         const double* scale, cudaStream_t st);
template <typename T>
void launch_batch_accum(const BatchInst* in, int ninst, int nblocks, double* u, const T* d, const double* scale,
                        cudaStream_t st);
// multigrid over a batch level
template <typename T>
void launch_batch_restrict(const BatchInst* in, int ninst, int nblocks, const T* rf, T* bc, const PcgScalars* s,
                           cudaStream_t st);
template <typename T>
void launch_batch_prolong_add(const BatchInst* in, int ninst, int nblocks, const T* xc, T* xf,
                              const PcgScalars* s, cudaStream_t st);
template <typename T>
void launch_batch_jacobi0(const BatchInst* in, int ninst, int nblocks, const T* fac, const ModalK<T>& K, int quirk,
                          T omega, const T* b, T* x, const PcgScalars* s, cudaStream_t st);
// x = A^-1 b with a dense symmetric n x n inverse (exact coarsest-level solve),
// for ncol right-hand sides n apart
template <typename T>
void launch_dense_coarse(long long n, const T* A, const T* b, T* x, const int* halt, cudaStream_t st,
                         int ncol = 1);
// one CTA per instance: iters Jacobi-PCG iterations on its coarsest grid
// (vectors and factors in shared memory when the largest grid, max_ndof /
// max_nelem, fits, with the element products in a shared scratch when that
// fits too; r, z, p, q, w are then unused)
template <typename T>
void launch_batch_coarse_pcg(const BatchInst* in, int ninst, const T* fac, const ModalK<T>& K, const T* dinv,
                             const T* b, T* x, T* r, T* z, T* p, T* q, T* w, int iters, const PcgScalars* s,
                             cudaStream_t st, long long max_ndof, long long max_nelem);
// Helmholtz matvec + p.Ap per instance over node vectors
template <typename T>
void launch_batch_helm_apply_dot(const BatchInst* in, int ninst, int nblocks, const HelmK& K, const T* x, T* y,
                                 const RedArgs& red, const PcgScalars* s, cudaStream_t st);

}  // namespace hexa
