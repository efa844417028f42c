// Stress post-processing of a solved displacement field: per element the
// centre-point strain and stress, von Mises, principal stresses and
// directions, the L1 norm of the principal stresses and (optionally) the Voigt
// stress vector.
//
// Restates Stress.stress_kernel! (src/Core/Stress.jl:159-285) on the
// structured grid: one thread per element, the 8 corner displacements read
// straight from the (FP64 or FP32) solution and rounded to Float32 as the
// reference's Float32.(U) (Stress.jl:291), the Jacobian formed from the node
// coordinates (i*dx, j*dy, k*dz) in Float32 as Mesh.generate_mesh's nodes
// (Mesh.jl:38) with the shape-function derivatives of the element centre,
// Hooke's law with E_loc = E * density (Stress.jl:183), and the principal
// stresses by 12 sweeps of cyclic Jacobi rotations (the published
// Jacobi eigenvalue method in the rotation form of Stress.jl:89-140),
// sorted descending.  Elements with density < 1e-6 get zeros (Stress.jl:165).
// Outputs are element-major: principal[3e + i], voigt[6e + i], dirs[3e + i].
#include <cuda_runtime.h>

#include <algorithm>

#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

namespace {

// One Jacobi rotation zeroing s_pq of the symmetric 3x3 (p < q, r the third
// index), applied to the eigenvector columns v[.][p], v[.][q].
__device__ __forceinline__ void jacobi_rotate(float& spp, float& sqq, float& spq, float& spr, float& sqr,
                                              float (&v)[3][3], int p, int q) {
  const float h = spq;
  const float g = 100.0f * fabsf(h);
  if (fabsf(spp) + g != fabsf(spp) || fabsf(sqq) + g != fabsf(sqq)) {
    const float theta = 0.5f * (sqq - spp) / h;
    float t = 1.0f / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
    if (theta < 0.0f) t = -t;
    const float c = 1.0f / sqrtf(t * t + 1.0f), s = t * c, tau = s / (1.0f + c);
    spp -= t * spq;
    sqq += t * spq;
    spq = 0.0f;
    const float tmp = spr;
    spr -= s * (sqr + tau * spr);
    sqr += s * (tmp - tau * sqr);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float vp = v[r][p];
      v[r][p] -= s * (v[r][q] + tau * vp);
      v[r][q] += s * (vp - tau * v[r][q]);
    }
  }
}

template <typename TU>
__global__ void stress_kernel(Grid g, const TU* __restrict__ u, const float* __restrict__ density, float E, float nu,
                              float dx, float dy, float dz, int save_voigt, float* __restrict__ principal,
                              float* __restrict__ vonmises, float* __restrict__ voigt, float* __restrict__ l1,
                              float* __restrict__ dmax, float* __restrict__ dmin) {
  const long long ne = g.nelem();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % g.nx);
    const long long t0 = e / g.nx;
    const int j = (int)(t0 % g.ny), k = (int)(t0 / g.ny);
    const float dens = density[e];
    if (dens < 1.0e-6f) {
#pragma unroll
      for (int q = 0; q < 3; ++q) principal[3 * e + q] = 0.f, dmax[3 * e + q] = 0.f, dmin[3 * e + q] = 0.f;
      vonmises[e] = 0.f;
      l1[e] = 0.f;
      if (save_voigt)
#pragma unroll
        for (int q = 0; q < 6; ++q) voigt[6 * e + q] = 0.f;
      continue;
    }
    const float Eloc = E * dens;
    // node a of the element in the reference's order n1..n8 (Mesh.jl:45-53)
    constexpr int DI[8] = {0, 1, 1, 0, 0, 1, 1, 0}, DJ[8] = {0, 0, 1, 1, 0, 0, 1, 1}, DK[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    float j11 = 0.f, j12 = 0.f, j13 = 0.f, j21 = 0.f, j22 = 0.f, j23 = 0.f, j31 = 0.f, j32 = 0.f, j33 = 0.f;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const float x = (float)(i + DI[a]) * dx, y = (float)(j + DJ[a]) * dy, z = (float)(k + DK[a]) * dz;
      const float nxi = DI[a] ? 0.125f : -0.125f, net = DJ[a] ? 0.125f : -0.125f, nze = DK[a] ? 0.125f : -0.125f;
      j11 += nxi * x; j12 += nxi * y; j13 += nxi * z;
      j21 += net * x; j22 += net * y; j23 += net * z;
      j31 += nze * x; j32 += nze * y; j33 += nze * z;
    }
    float det = j11 * (j22 * j33 - j23 * j32) - j12 * (j21 * j33 - j23 * j31) + j13 * (j21 * j32 - j22 * j31);
    if (det <= 1.0e-12f) det = 1.0f;
    const float id = 1.0f / det;
    const float a11 = (j22 * j33 - j23 * j32) * id, a12 = -(j12 * j33 - j13 * j32) * id, a13 = (j12 * j23 - j13 * j22) * id;
    const float a21 = -(j21 * j33 - j23 * j31) * id, a22 = (j11 * j33 - j13 * j31) * id, a23 = -(j11 * j23 - j13 * j21) * id;
    const float a31 = (j21 * j32 - j22 * j31) * id, a32 = -(j11 * j32 - j12 * j31) * id, a33 = (j11 * j22 - j12 * j21) * id;
    float exx = 0.f, eyy = 0.f, ezz = 0.f, gxy = 0.f, gyz = 0.f, gxz = 0.f;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const long long n = (long long)(i + DI[a]) + (long long)g.NX * ((long long)(j + DJ[a]) + (long long)g.NY * (k + DK[a]));
      const float ux = (float)u[3 * n], uy = (float)u[3 * n + 1], uz = (float)u[3 * n + 2];
      const float nxi = DI[a] ? 0.125f : -0.125f, net = DJ[a] ? 0.125f : -0.125f, nze = DK[a] ? 0.125f : -0.125f;
      const float ddx = nxi * a11 + net * a21 + nze * a31;
      const float ddy = nxi * a12 + net * a22 + nze * a32;
      const float ddz = nxi * a13 + net * a23 + nze * a33;
      exx += ddx * ux;
      eyy += ddy * uy;
      ezz += ddz * uz;
      gxy += ddy * ux + ddx * uy;
      gyz += ddz * uy + ddy * uz;
      gxz += ddz * ux + ddx * uz;
    }
    const float fact = Eloc / ((1.0f + nu) * (1.0f - 2.0f * nu));
    const float c1 = (1.0f - nu) * fact, c2 = nu * fact, c3 = (0.5f - nu) * fact;
    const float sxx = c1 * exx + c2 * eyy + c2 * ezz;
    const float syy = c2 * exx + c1 * eyy + c2 * ezz;
    const float szz = c2 * exx + c2 * eyy + c1 * ezz;
    const float sxy = c3 * gxy, syz = c3 * gyz, sxz = c3 * gxz;
    if (save_voigt) {
      voigt[6 * e] = sxx, voigt[6 * e + 1] = syy, voigt[6 * e + 2] = szz;
      voigt[6 * e + 3] = sxy, voigt[6 * e + 4] = syz, voigt[6 * e + 5] = sxz;
    }
    const float vm2 = 0.5f * ((sxx - syy) * (sxx - syy) + (syy - szz) * (syy - szz) + (szz - sxx) * (szz - sxx)) +
                      3.0f * (sxy * sxy + syz * syz + sxz * sxz);
    vonmises[e] = sqrtf(fmaxf(0.0f, vm2));
    // eigenpairs: cyclic Jacobi, at most 12 sweeps of the (1,2), (1,3), (2,3) rotations
    float s11 = sxx, s22 = syy, s33 = szz, s12 = sxy, s23 = syz, s13 = sxz;
    float v[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
    for (int it = 0; it < 12; ++it) {
      if (fmaxf(fabsf(s12), fmaxf(fabsf(s23), fabsf(s13))) < 1.0e-9f) break;
      jacobi_rotate(s11, s22, s12, s13, s23, v, 0, 1);
      jacobi_rotate(s11, s33, s13, s12, s23, v, 0, 2);
      jacobi_rotate(s22, s33, s23, s12, s13, v, 1, 2);
    }
    // descending order, columns of v swapped with their eigenvalues
    auto swapcol = [&](int p, int q) {
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float t = v[r][p];
        v[r][p] = v[r][q];
        v[r][q] = t;
      }
    };
    if (s11 < s22) { const float t = s11; s11 = s22; s22 = t; swapcol(0, 1); }
    if (s22 < s33) { const float t = s22; s22 = s33; s33 = t; swapcol(1, 2); }
    if (s11 < s22) { const float t = s11; s11 = s22; s22 = t; swapcol(0, 1); }
    principal[3 * e] = s11, principal[3 * e + 1] = s22, principal[3 * e + 2] = s33;
#pragma unroll
    for (int r = 0; r < 3; ++r) dmax[3 * e + r] = v[r][0], dmin[3 * e + r] = v[r][2];
    l1[e] = fabsf(s11) + fabsf(s22) + fabsf(s33);
  }
}

}  // namespace

template <typename TU>
void launch_stress(const Grid& g, const TU* u, const float* density, float E, float nu, float dx, float dy, float dz,
                   int save_voigt, float* principal, float* vonmises, float* voigt, float* l1, float* dmax,
                   float* dmin, cudaStream_t st) {
  const long long ne = g.nelem();
  const int blocks = (int)std::max<long long>(1, std::min<long long>((ne + 255) / 256, 152LL * 16));
  stress_kernel<TU><<<blocks, 256, 0, st>>>(g, u, density, E, nu, dx, dy, dz, save_voigt, principal, vonmises, voigt,
                                            l1, dmax, dmin);
}

template void launch_stress<double>(const Grid&, const double*, const float*, float, float, float, float, float, int,
                                    float*, float*, float*, float*, float*, float*, cudaStream_t);
template void launch_stress<float>(const Grid&, const float*, const float*, float, float, float, float, float, int,
                                   float*, float*, float*, float*, float*, float*, cudaStream_t);

}  // namespace hexa
