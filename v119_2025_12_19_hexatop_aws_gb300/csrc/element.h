// Host-side element matrices (see element.cpp).
#pragma once
#include "hexa_common.cuh"

namespace hexa {

// 24x24 column-major K0 for E = 1 (Element.jl:104-111); 0 ok, <0 error.
int canonical_stiffness(double dx, double dy, double dz, double nu, double* ke);
// 8x8 column-major Laplacian and mass (Element.jl:113-134).
int scalar_matrices(double dx, double dy, double dz, int quirk, double* Ke, double* Me);
// Hadamard-basis blocks of K0; fails (-3) if K0 is not block diagonal in that
// basis to 1e-12 relative (max_dropped receives the largest dropped entry).
int modal_blocks(const double* ke, ModalK<double>* out, double* max_dropped);
// Upper bound of lambda_max(D^-1 (K + sigma I)) for any non-negative element
// factors: max over one element of lambda_max(D0^-1/2 K0 D0^-1/2), D0 the
// diagonal the smoother uses (quirk: x-diagonal for every component).
double smoother_bound(const double* ke, int quirk);
// R^2 Ke + Me permuted from n1..n8 order to corner order dx + 2dy + 4dz.
void helm_corner_matrix(const double* Ke, const double* Me, double R, double A[8][8]);

}  // namespace hexa
