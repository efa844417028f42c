// Host-side element matrices.
//
// canonical_stiffness follows Element.get_canonical_stiffness /
// hex_element_stiffness / material_matrix / shape_functions
// (src/Core/Element.jl:23-111): brick centred at the origin, E = 1,
// 2x2x2 Gauss points +-1/sqrt(3), ke += B^T D B detJ, Voigt order
// (xx, yy, zz, xy, yz, xz) with engineering shears.  It is evaluated in FP64;
// the reference evaluates the same formulas in Float32 and promotes
// (GPUSolver.jl:248-249), a difference below 2e-7 relative.
//
// scalar_matrices follows Element.get_scalar_canonical_matrices
// (Element.jl:113-134), including the reference's top-face z = +dz (quirk=1).
//
// modal_blocks builds the Hadamard-basis blocks the GPU operator uses.
#include "element.h"

#include <cmath>
#include <cstring>

namespace hexa {

// Natural coordinates of n1..n8 (Element.jl:8-17).
static const double kNat[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                  {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

static void shape(double xi, double eta, double zeta, double N[8], double dN[8][3]) {
  for (int i = 0; i < 8; ++i) {
    const double tx = 1.0 + xi * kNat[i][0], ty = 1.0 + eta * kNat[i][1], tz = 1.0 + zeta * kNat[i][2];
    N[i] = 0.125 * tx * ty * tz;
    dN[i][0] = 0.125 * kNat[i][0] * ty * tz;
    dN[i][1] = 0.125 * tx * kNat[i][1] * tz;
    dN[i][2] = 0.125 * tx * ty * kNat[i][2];
  }
}

static double det3(const double J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

static void inv3(const double J[3][3], double d, double Ji[3][3]) {
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
}

// dN/dx at one Gauss point for the element with the given nodal coordinates.
static bool grad_at(const double nodes[8][3], double xi, double eta, double zeta, double N[8],
                    double dNdx[8][3], double* detJ) {
  double dN[8][3];
  shape(xi, eta, zeta, N, dN);
  double J[3][3] = {{0}};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int i = 0; i < 8; ++i) J[a][b] += dN[i][a] * nodes[i][b];
  const double d = det3(J);
  if (!(d > 0.0)) return false;  // Element.jl:84-86 "Non-positive Jacobian"
  double Ji[3][3];
  inv3(J, d, Ji);
  for (int i = 0; i < 8; ++i)
    for (int a = 0; a < 3; ++a) {
      double s = 0.0;
      for (int b = 0; b < 3; ++b) s += dN[i][b] * Ji[a][b];  // dN * inv(J)^T
      dNdx[i][a] = s;
    }
  *detJ = d;
  return true;
}

int canonical_stiffness(double dx, double dy, double dz, double nu, double* ke) {
  if (!(dx > 0 && dy > 0 && dz > 0) || !(nu > -1.0 && nu < 0.5)) return -1;
  double nodes[8][3] = {{0, 0, 0}, {dx, 0, 0}, {dx, dy, 0}, {0, dy, 0}, {0, 0, dz}, {dx, 0, dz}, {dx, dy, dz}, {0, dy, dz}};
  for (int i = 0; i < 8; ++i) {
    nodes[i][0] -= dx / 2;
    nodes[i][1] -= dy / 2;
    nodes[i][2] -= dz / 2;
  }
  // material_matrix (Element.jl:45-71), E = 1
  const double f = 1.0 / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double c1 = (1.0 - nu) * f, c2 = nu * f, c3 = ((1.0 - 2.0 * nu) / 2.0) * f;
  double D[6][6] = {{0}};
  D[0][0] = D[1][1] = D[2][2] = c1;
  D[0][1] = D[0][2] = D[1][0] = D[1][2] = D[2][0] = D[2][1] = c2;
  D[3][3] = D[4][4] = D[5][5] = c3;
  std::memset(ke, 0, sizeof(double) * 576);
  const double a = 1.0 / std::sqrt(3.0);
  const double gp[2] = {-a, a};
  for (int ix = 0; ix < 2; ++ix)
    for (int iy = 0; iy < 2; ++iy)
      for (int iz = 0; iz < 2; ++iz) {
        double N[8], G[8][3], detJ;
        if (!grad_at(nodes, gp[ix], gp[iy], gp[iz], N, G, &detJ)) return -2;
        double B[6][24] = {{0}};
        for (int i = 0; i < 8; ++i) {
          const int o = 3 * i;
          B[0][o] = G[i][0];
          B[1][o + 1] = G[i][1];
          B[2][o + 2] = G[i][2];
          B[3][o] = G[i][1];
          B[3][o + 1] = G[i][0];
          B[4][o + 1] = G[i][2];
          B[4][o + 2] = G[i][1];
          B[5][o] = G[i][2];
          B[5][o + 2] = G[i][0];
        }
        double DB[6][24];
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int t = 0; t < 6; ++t) s += D[r][t] * B[t][c];
            DB[r][c] = s;
          }
        for (int r = 0; r < 24; ++r)
          for (int c = 0; c < 24; ++c) {
            double s = 0.0;
            for (int t = 0; t < 6; ++t) s += B[t][r] * DB[t][c];
            ke[r + 24 * c] += s * detJ;  // column-major
          }
      }
  return 0;
}

int scalar_matrices(double dx, double dy, double dz, int quirk, double* Ke, double* Me) {
  if (!(dx > 0 && dy > 0 && dz > 0)) return -1;
  const double ztop = quirk ? dz : dz / 2;
  const double nodes[8][3] = {{-dx / 2, -dy / 2, -dz / 2}, {dx / 2, -dy / 2, -dz / 2}, {dx / 2, dy / 2, -dz / 2},
                              {-dx / 2, dy / 2, -dz / 2},  {-dx / 2, -dy / 2, ztop},   {dx / 2, -dy / 2, ztop},
                              {dx / 2, dy / 2, ztop},      {-dx / 2, dy / 2, ztop}};
  std::memset(Ke, 0, sizeof(double) * 64);
  std::memset(Me, 0, sizeof(double) * 64);
  const double a = 1.0 / std::sqrt(3.0);
  const double gp[2] = {-a, a};
  for (int ix = 0; ix < 2; ++ix)
    for (int iy = 0; iy < 2; ++iy)
      for (int iz = 0; iz < 2; ++iz) {
        double N[8], G[8][3], detJ;
        if (!grad_at(nodes, gp[ix], gp[iy], gp[iz], N, G, &detJ)) return -2;
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) {
            Ke[r + 8 * c] += (G[r][0] * G[c][0] + G[r][1] * G[c][1] + G[r][2] * G[c][2]) * detJ;
            Me[r + 8 * c] += N[r] * N[c] * detJ;
          }
      }
  return 0;
}

// Corner index (dx + 2dy + 4dz) of the reference's local node n1..n8.
static const int kRefToCorner[8] = {0, 1, 3, 2, 4, 5, 7, 6};

static bool modal_structural_nz(int q, int c, int c2) {
  if (q == 1 || q == 2 || q == 4) {
    const int c0 = (q == 1) ? 0 : (q == 2 ? 1 : 2);
    return c != c0 && c2 != c0;
  }
  if (q == 3 || q == 5 || q == 6) {
    const int cf = (q == 3) ? 2 : (q == 5 ? 1 : 0);
    return (c == cf) == (c2 == cf);
  }
  return true;
}

int modal_blocks(const double* ke, ModalK<double>* out, double* max_dropped) {
  // H[m][corner] = prod_d s_d^{m_d}, s_d = -1 (low) / +1 (high)
  double H[8][8];
  for (int m = 0; m < 8; ++m)
    for (int cc = 0; cc < 8; ++cc) {
      double v = 1.0;
      for (int d = 0; d < 3; ++d)
        if ((m >> d) & 1) v *= ((cc >> d) & 1) ? 1.0 : -1.0;
      H[m][cc] = v;
    }
  // M'[(m,c),(m2,c2)] = sum_{n,n2} H[m][n] K[(n,c),(n2,c2)] H[m2][n2] / 64
  double M[24][24];
  double kmax = 0.0;
  for (int i = 0; i < 576; ++i) kmax = std::fmax(kmax, std::fabs(ke[i]));
  for (int m = 0; m < 8; ++m)
    for (int c = 0; c < 3; ++c)
      for (int m2 = 0; m2 < 8; ++m2)
        for (int c2 = 0; c2 < 3; ++c2) {
          double s = 0.0;
          for (int n = 0; n < 8; ++n)
            for (int n2 = 0; n2 < 8; ++n2) {
              const int r = 3 * n + c, col = 3 * n2 + c2;  // reference DOF order
              s += H[m][kRefToCorner[n]] * ke[r + 24 * col] * H[m2][kRefToCorner[n2]];
            }
          M[3 * m + c][3 * m2 + c2] = s / 64.0;
        }
  double dropped = 0.0;
  for (int i = 0; i < 24; ++i)
    for (int j = 0; j < 24; ++j) {
      const int q1 = (i / 3) ^ (1 << (i % 3)), q2 = (j / 3) ^ (1 << (j % 3));
      if (q1 != q2) dropped = std::fmax(dropped, std::fabs(M[i][j]));
    }
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c)
      for (int c2 = 0; c2 < 3; ++c2) {
        const double v = M[3 * (q ^ (1 << c)) + c][3 * (q ^ (1 << c2)) + c2];
        if (modal_structural_nz(q, c, c2)) {
          out->B[q][c][c2] = v;
        } else {
          dropped = std::fmax(dropped, std::fabs(v));
          out->B[q][c][c2] = 0.0;
        }
      }
  for (int c = 0; c < 3; ++c) out->dd[c] = ke[c + 24 * c];
  if (max_dropped) *max_dropped = dropped / (kmax > 0 ? kmax : 1.0);
  return (dropped <= 1e-12 * kmax) ? 0 : -3;
}

double smoother_bound(const double* ke, int quirk) {
  double S[24][24];
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c) {
      const double dr = quirk ? ke[(3 * (r / 3)) * 25] : ke[r * 25];
      const double dc = quirk ? ke[(3 * (c / 3)) * 25] : ke[c * 25];
      S[r][c] = ke[r + 24 * c] / std::sqrt(dr * dc);
    }
  // power iteration on the symmetric positive semidefinite S
  double v[24], w[24], lam = 0.0;
  for (int i = 0; i < 24; ++i) v[i] = 1.0 + 0.01 * i * ((i & 1) ? -1 : 1);
  for (int it = 0; it < 500; ++it) {
    double nrm = 0.0;
    for (int i = 0; i < 24; ++i) {
      double t = 0.0;
      for (int j = 0; j < 24; ++j) t += S[i][j] * v[j];
      w[i] = t;
      nrm += t * t;
    }
    nrm = std::sqrt(nrm);
    if (nrm == 0.0) break;
    double num = 0.0;
    for (int i = 0; i < 24; ++i) num += v[i] * w[i];
    double vv = 0.0;
    for (int i = 0; i < 24; ++i) vv += v[i] * v[i];
    lam = num / vv;
    for (int i = 0; i < 24; ++i) v[i] = w[i] / nrm;
  }
  return lam;
}

void helm_corner_matrix(const double* Ke, const double* Me, double R, double A[8][8]) {
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < 8; ++c)
      A[kRefToCorner[r]][kRefToCorner[c]] = R * R * Ke[r + 8 * c] + Me[r + 8 * c];
}

}  // namespace hexa
