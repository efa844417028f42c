// Shared device-side definitions of the hex8 solve path.
//
// Grid layout (structured brick, src/Mesh/Mesh.jl:23-60, 0-based here):
//   node (i,j,k)    -> n = i + NX*(j + NY*k),   NX = nx+1, NY = ny+1, NZ = nz+1
//   element (i,j,k) -> e = i + nx*(j + ny*k)
//   vectors are AoS xyz per node: dof = 3*n + c   (GPUSolver.jl:100-108)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hexa {

struct Grid {
  int nx, ny, nz;  // elements
  int NX, NY, NZ;  // nodes
  __host__ __device__ long long nnode() const { return (long long)NX * NY * NZ; }
  __host__ __device__ long long nelem() const { return (long long)nx * ny * nz; }
  __host__ __device__ long long ndof() const { return 3LL * NX * NY * NZ; }
};

inline Grid make_grid(int nx, int ny, int nz) {
  Grid g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.NX = nx + 1; g.NY = ny + 1; g.NZ = nz + 1;
  return g;
}

// Dirichlet set: face clamps (all three DOFs of every node on the face) OR-ed
// with an optional per-node bit mask (bit c set = component c fixed).
struct Mask {
  uint32_t faces;
  const uint8_t* node;
};

__device__ __forceinline__ unsigned fixed_bits(const Grid& g, const Mask& m, int i, int j, int k,
                                               long long n) {
  unsigned f = 0;
  const uint32_t F = m.faces;
  if (F) {
    if (((F & 1u) && i == 0) || ((F & 2u) && i == g.NX - 1) || ((F & 4u) && j == 0) ||
        ((F & 8u) && j == g.NY - 1) || ((F & 16u) && k == 0) || ((F & 32u) && k == g.NZ - 1))
      f = 7u;
  }
  if (m.node) f |= (unsigned)__ldg(m.node + n);
  return f;
}

// K0 in the per-element Hadamard basis.  With phi_m(node) = prod_d s_d^{m_d}
// (s_d = -1 on the low face, +1 on the high face) and u_hat = H u per
// component, the 24x24 K0 is block diagonal: component c of mode m couples
// only within the class q = m ^ (1<<c), giving eight 3x3 blocks
//   w_hat[m][c] = sum_c' B[q][c][c'] * u_hat[q ^ (1<<c')][c'],
// and w = H^T w_hat.  B carries the 1/64 of H^T H = 8 I on both sides.
// dd[c] is the K0 diagonal entry of component c (equal for all 8 nodes).
template <typename T>
struct ModalK {
  T B[8][3][3];
  T dd[3];
};

// Device-resident PCG scalars.  Kernels read them (coefficients, halt flag);
// the last block of a reducing kernel updates them (see finalize()).
struct PcgScalars {
  double rz;        // r . z of the current iteration
  double rz_prev;   // r . z_old (flexible beta)
  double pAp;
  double alpha;
  double beta;
  double rr;        // ||r||^2 of the recursive residual
  double bnorm;     // ||b||
  double relres;    // sqrt(rr)/bnorm at the last test
  double best_rel;
  double tol;
  double dtmp[6];   // scratch reduction results
  int halt;         // nonzero: every kernel of the iteration returns at once
  int status;       // 0 running, 1 converged, 2 nan/inf, 3 diverged, 4 breakdown (|pAp|<1e-20)
  int iter;         // completed iterations
  int max_iter;
  int cadence;      // test convergence when iter==1 or iter%cadence==0
  int test_now;
  int no_div;       // 1: no divergence test (the filter loop has none)
  int pad;
};

enum FinalizeOp {
  FIN_NONE = 0,
  FIN_STORE = 1,        // dst = sum
  FIN_PCG_ALPHA = 2,    // pAp = sum; alpha = rz/pAp; breakdown test
  FIN_PCG_RES = 3,      // rr = sum0; (rz_new = sum1 if two sums) ; convergence test, iter++
  FIN_PCG_BETA = 4,     // rz_new = sum0 [, rz_old_mix = sum1]; beta
  FIN_INIT_RES = 5,     // rr = sum0 ; relres
  FIN_INIT_RZ = 6,      // rz = sum0
  FIN_BLOCK_RES = 7,    // nsum column norms ||R_j||^2 (to dst when given); rr = max; test, iter++
  FIN_PCG_RES_MG = 8,   // FIN_PCG_RES with sum1 = r_new.z_old kept for FIN_PCG_BETA_RZ
  FIN_PCG_BETA_RZ = 9,  // rz_new = sum0; flexible beta = (rz_new - r_new.z_old) / rz
};

// Reduction plumbing of one reducing launch: per-block partials, a ticket
// counter and what the last block does with the total.
// With ncol > 1 the launch solves ncol independent columns (right-hand
// sides): block b belongs to column b % ncol, each column has its own ticket,
// scalars (s + col) and destination (dst + col * nsum), and the grid size is a
// multiple of ncol.
struct RedArgs {
  double* partials;     // [nblocks * nsum]
  unsigned* ticket;     // [ncol], zero before the launch, reset by the column's last block
  double* dst;          // FIN_STORE destination (nsum values per column)
  PcgScalars* s;        // scalars for FIN_PCG_* (one per column)
  int op;
  int nsum;             // 1 or 2 sums per thread
  int ncol = 1;         // columns of a batched pass (block b works on column b % ncol)
};

// Halt flag of column col given the flag of column 0 (flags live in an array
// of PcgScalars).
__device__ __forceinline__ bool halted(const int* halt0, int col) {
  return halt0 && *((volatile const int*)((const char*)halt0 + (size_t)col * sizeof(PcgScalars)));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void finalize_scalars(const RedArgs& r, const double* tot, int col) {
  PcgScalars* s = r.s ? r.s + col : nullptr;
  switch (r.op) {
    case FIN_STORE:
      for (int q = 0; q < r.nsum; ++q) r.dst[col * r.nsum + q] = tot[q];
      break;
    case FIN_PCG_ALPHA: {
      s->pAp = tot[0];
      // GPUSolver.jl:374 stops on the absolute test |p.Ap| < 1e-20, which ends
      // tight solves of unit-load problems early; for the SPD (K + sigma I)
      // only non-positive (or NaN) curvature is a breakdown here.
      if (!(tot[0] > 0.0)) {
        s->status = 4;
        s->halt = 1;
        s->alpha = 0.0;
      } else {
        s->alpha = s->rz / tot[0];
      }
      break;
    }
    case FIN_PCG_RES_MG:
      s->dtmp[0] = tot[1];
      [[fallthrough]];
    case FIN_PCG_RES: {
      s->rr = tot[0];
      s->iter += 1;
      const int k = s->iter;
      // cadence > 0: test at k == 1 and every cadence iterations (GPUSolver.jl:379);
      // cadence < 0: only every |cadence| iterations (GPUHelmholtz.jl:245); 0: never
      const int cad = s->cadence;
      const bool test = (cad > 0) ? ((cad == 1) || (k == 1) || (k % cad == 0)) : ((cad < 0) && (k % (-cad) == 0));
      s->test_now = test ? 1 : 0;
      if (r.op == FIN_PCG_RES && r.nsum > 1) {  // Jacobi fused: rz_new available now
        s->rz_prev = s->rz;
        s->beta = (s->rz != 0.0) ? tot[1] / s->rz : 0.0;
        s->rz = tot[1];
      }
      if (test) {
        const double rel = sqrt(fmax(tot[0], 0.0)) / s->bnorm;
        s->relres = rel;
        if (!(rel == rel) || isinf(rel)) {
          s->status = 2; s->halt = 1;
        } else if (rel < s->tol) {
          s->status = 1; s->halt = 1;
        } else if (!s->no_div && (rel > 10.0 || (k > 500 && rel > s->best_rel * 100.0))) {  // GPUSolver.jl:397
          s->status = 3; s->halt = 1;
        }
        if (rel < s->best_rel) s->best_rel = rel;
      }
      if (!s->halt && k >= s->max_iter) s->halt = 1;
      break;
    }
    case FIN_PCG_BETA: {
      // tot[0] = r.z_new ; tot[1] (flexible) = r.z_old
      const double rz_new = tot[0];
      const double num = (r.nsum > 1) ? (rz_new - tot[1]) : rz_new;
      s->beta = (s->rz != 0.0) ? num / s->rz : 0.0;
      s->rz_prev = s->rz;
      s->rz = rz_new;
      break;
    }
    case FIN_PCG_BETA_RZ: {
      const double rz_new = tot[0];
      s->beta = (s->rz != 0.0) ? (rz_new - s->dtmp[0]) / s->rz : 0.0;
      s->rz_prev = s->rz;
      s->rz = rz_new;
      break;
    }
    case FIN_INIT_RES: {
      s->rr = tot[0];
      s->relres = sqrt(fmax(tot[0], 0.0)) / s->bnorm;
      break;
    }
    case FIN_INIT_RZ:
      s->rz = tot[0];
      break;
    case FIN_BLOCK_RES: {
      double mx = 0.0;
      bool bad = false;
      for (int q = 0; q < r.nsum; ++q) {
        if (r.dst) r.dst[q] = tot[q];
        if (!(tot[q] == tot[q]) || isinf(tot[q])) bad = true;
        mx = fmax(mx, tot[q]);
      }
      s->rr = mx;
      s->iter += 1;
      const double rel = sqrt(mx) / s->bnorm;
      s->relres = rel;
      if (bad) {
        s->status = 2; s->halt = 1;
      } else if (rel < s->tol) {
        s->status = 1; s->halt = 1;
      }
      if (rel < s->best_rel) s->best_rel = rel;
      if (!s->halt && s->iter >= s->max_iter) s->halt = 1;
      break;
    }
    default:
      break;
  }
}

// Block reduction of nsum values per thread, then the last block (by ticket)
// of the same reduction group sums the per-block partials in block order and
// runs the finalize op.  The order of every addition is fixed, so results are
// bitwise reproducible.  A group is column `col` of the scalars/tickets; its
// nb blocks have partial slots base, base + step, ..., this block's slot is bid.
template <int NSUM>
__device__ __forceinline__ void block_reduce_finalize_at(const RedArgs& r, double (&v)[NSUM], int col, long long bid,
                                                         long long nb, long long base, long long step) {
  __shared__ double sred[NSUM][32];
  __shared__ bool am_last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, wid = tid >> 5, nw = (nthr + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NSUM; ++q) {
    double t = warp_sum(v[q]);
    if (lane == 0) sred[q][wid] = t;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NSUM; ++q) {
      double t = (lane < nw) ? sred[q][lane] : 0.0;
      t = warp_sum(t);
      if (lane == 0) r.partials[bid * NSUM + q] = t;
    }
    if (lane == 0) {
      __threadfence();
      unsigned tk = atomicAdd(r.ticket + col, 1u);
      am_last = (tk == (unsigned)(nb - 1));
    }
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  // last block: fixed-order sum over partials
  double acc[NSUM];
#pragma unroll
  for (int q = 0; q < NSUM; ++q) acc[q] = 0.0;
  for (long long b = tid; b < nb; b += nthr) {
#pragma unroll
    for (int q = 0; q < NSUM; ++q) acc[q] += ((volatile double*)r.partials)[(base + b * step) * NSUM + q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NSUM; ++q) {
    double t = warp_sum(acc[q]);
    if (lane == 0) sred[q][wid] = t;
  }
  __syncthreads();
  if (tid == 0) {
    double tot[NSUM];
#pragma unroll
    for (int q = 0; q < NSUM; ++q) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += sred[q][w];
      tot[q] = t;
    }
    finalize_scalars(r, tot, col);
    r.ticket[col] = 0u;
  }
}

// The whole grid is one group per column (block b works on column b % ncol).
template <int NSUM>
__device__ __forceinline__ void block_reduce_finalize(const RedArgs& r, double (&v)[NSUM]) {
  const long long bid = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
  const long long nball = (long long)gridDim.x * gridDim.y * gridDim.z;
  const int ncol = r.ncol > 1 ? r.ncol : 1;
  const int col = (int)(bid % ncol);
  block_reduce_finalize_at<NSUM>(r, v, col, bid, nball / ncol, col, ncol);
}

}  // namespace hexa
