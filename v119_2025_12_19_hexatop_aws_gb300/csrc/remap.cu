// Density and thermal-field transfer onto a refined grid: one thread per new
// element, its centroid mapped into the old grid's continuous cell-index
// space, the old cell-centred density interpolated trilinearly (clamped to the
// outer cell centres) and, in the "hard" update, projected (> 0.4 -> 1,
// < 0.2 -> 1e-4); the thermal field takes the value of the lower-corner old
// cell.  Restates MeshRefiner.refine_mesh_and_fields' mapping loop
// (src/Mesh/MeshRefiner.jl:188-240) and interpolate_trilinear_projected
// (:45-74) in Float32.
#include <cuda_runtime.h>

#include <algorithm>

#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

namespace {

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ long long clampl(long long v, long long lo, long long hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void remap_kernel(int onx, int ony, int onz, int nnx, int nny, int nnz, float ndx, float ndy, float ndz,
                             float lx, float ly, float lz, int projection, const float* __restrict__ dens,
                             const float* __restrict__ alpha, float* __restrict__ nd, float* __restrict__ na) {
  const long long n = (long long)nnx * nny * nnz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long ix = e % nnx + 1, rem = e / nnx, iy = rem % nny + 1, iz = rem / nny + 1;  // 1-based
    const float cx = __fmul_rn((float)ix - 0.5f, ndx), cy = __fmul_rn((float)iy - 0.5f, ndy);
    const float cz = __fmul_rn((float)iz - 0.5f, ndz);
    const float u = clampf(__fmul_rn(__fdiv_rn(cx, lx), (float)onx), 0.5f, (float)onx - 0.5f);
    const float v = clampf(__fmul_rn(__fdiv_rn(cy, ly), (float)ony), 0.5f, (float)ony - 0.5f);
    const float w = clampf(__fmul_rn(__fdiv_rn(cz, lz), (float)onz), 0.5f, (float)onz - 0.5f);
    const long long u0 = (long long)floorf(u - 0.5f), v0 = (long long)floorf(v - 0.5f), w0 = (long long)floorf(w - 0.5f);
    const float tx = clampf((u - 0.5f) - (float)u0, 0.f, 1.f);
    const float ty = clampf((v - 0.5f) - (float)v0, 0.f, 1.f);
    const float tz = clampf((w - 0.5f) - (float)w0, 0.f, 1.f);
    // clamped neighbours, 0-based
    const long long i0 = clampl(u0, 0, onx - 1), i1 = clampl(u0 + 1, 0, onx - 1);
    const long long j0 = clampl(v0, 0, ony - 1), j1 = clampl(v0 + 1, 0, ony - 1);
    const long long k0 = clampl(w0, 0, onz - 1), k1 = clampl(w0 + 1, 0, onz - 1);
    const long long sx = onx, sxy = (long long)onx * ony;
    auto at = [&](long long i, long long j, long long k) { return dens[i + sx * j + sxy * k]; };
    // no contraction into FMAs: the reference evaluates each product and sum rounded
    auto lerp = [](float a, float b, float t) { return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t)); };
    const float c00 = lerp(at(i0, j0, k0), at(i1, j0, k0), tx);
    const float c10 = lerp(at(i0, j1, k0), at(i1, j1, k0), tx);
    const float c01 = lerp(at(i0, j0, k1), at(i1, j0, k1), tx);
    const float c11 = lerp(at(i0, j1, k1), at(i1, j1, k1), tx);
    const float c0 = lerp(c00, c10, ty), c1 = lerp(c01, c11, ty);
    float val = lerp(c0, c1, tz);
    if (projection) val = val > 0.4f ? 1.0f : (val < 0.2f ? 0.0001f : val);
    nd[e] = val;
    if (na) na[e] = alpha ? alpha[i0 + sx * j0 + sxy * k0] : 0.f;
  }
}

// Nodal displacements carried onto the grown grid as a warm start: new node
// (i, j, k) sits at old node-index coordinates (i * onx / nnx, ...), both
// grids spanning the same box; the three components are interpolated
// trilinearly from the 8 surrounding old nodes in FP64.  The reference resets
// U to zero after a refinement (Main.jl:412-413); this transfer only changes
// the first guess of the next solve, not its answer.
__global__ void remap_nodal_kernel(int onx, int ony, int onz, int nnx, int nny, int nnz, const double* __restrict__ u,
                                   double* __restrict__ un) {
  const long long NX = nnx + 1, NY = nny + 1, n = NX * NY * (long long)(nnz + 1);
  const long long OX = onx + 1, OXY = (long long)(onx + 1) * (ony + 1);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long long i = q % NX, rem = q / NX, j = rem % NY, k = rem / NY;
    auto axis = [](long long idx, int on, int nn, int* i0, double* t) {
      const double sc = fmin(fmax((double)idx * (double)on / (double)nn, 0.0), (double)on);
      int a = (int)floor(sc);
      a = a > on - 1 ? on - 1 : (a < 0 ? 0 : a);
      *i0 = a;
      *t = sc - (double)a;
    };
    int i0, j0, k0;
    double tx, ty, tz;
    axis(i, onx, nnx, &i0, &tx);
    axis(j, ony, nny, &j0, &ty);
    axis(k, onz, nnz, &k0, &tz);
    const long long base = i0 + OX * j0 + OXY * k0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      auto at = [&](int di, int dj, int dk) { return u[3 * (base + di + OX * dj + OXY * dk) + c]; };
      const double c00 = at(0, 0, 0) * (1.0 - tx) + at(1, 0, 0) * tx;
      const double c10 = at(0, 1, 0) * (1.0 - tx) + at(1, 1, 0) * tx;
      const double c01 = at(0, 0, 1) * (1.0 - tx) + at(1, 0, 1) * tx;
      const double c11 = at(0, 1, 1) * (1.0 - tx) + at(1, 1, 1) * tx;
      const double c0 = c00 * (1.0 - ty) + c10 * ty, c1 = c01 * (1.0 - ty) + c11 * ty;
      un[3 * q + c] = c0 * (1.0 - tz) + c1 * tz;
    }
  }
}

}  // namespace

void launch_remap_nodal(int onx, int ony, int onz, int nnx, int nny, int nnz, const double* u, double* un,
                        cudaStream_t st) {
  const long long n = (long long)(nnx + 1) * (nny + 1) * (nnz + 1);
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16));
  remap_nodal_kernel<<<blocks, 256, 0, st>>>(onx, ony, onz, nnx, nny, nnz, u, un);
}

void launch_remap(int onx, int ony, int onz, int nnx, int nny, int nnz, float ndx, float ndy, float ndz, float lx,
                  float ly, float lz, int projection, const float* dens, const float* alpha, float* nd, float* na,
                  cudaStream_t st) {
  const long long n = (long long)nnx * nny * nnz;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16));
  remap_kernel<<<blocks, 256, 0, st>>>(onx, ony, onz, nnx, nny, nnz, ndx, ndy, ndz, lx, ly, lz, projection, dens,
                                       alpha, nd, na);
}

}  // namespace hexa
