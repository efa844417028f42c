"""Generates tests/golden/element_kat.json: exact element matrices.

The reference has no tests or golden vectors, and Julia is not available to
run it, so the oracle's element matrices are pinned against exact rational
integrals computed here with fractions.Fraction, independently of any
quadrature.  For trilinear hex8 bricks the integrands are polynomials of
degree <= 2 per axis, which the reference's 2x2x2 Gauss rule
(src/Core/Element.jl:73-102, 113-134) integrates exactly, so the reference's
matrices equal these up to rounding.

  K0[(a,c),(b,d)] = int lam dN_a/dx_c dN_b/dx_d
                  + mu (delta_cd grad N_a . grad N_b + dN_a/dx_d dN_b/dx_c)
  Ke[a,b] = int grad N_a . grad N_b,   Me[a,b] = int N_a N_b

over the brick [0,hx]x[0,hy]x[0,hz]; node order n1..n8 of Element.jl:8-17;
DOF order node-major xyz; E = 1.  The Helmholtz "quirk" brick has height
1.5*dz (the reference's top face at +dz, Element.jl:116).

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
from fractions import Fraction as F
from pathlib import Path

NODES = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def one_d(h):
    M = [[h / 3, h / 6], [h / 6, h / 3]]           # int phi_a phi_b
    D = [[1 / h, -1 / h], [-1 / h, 1 / h]]         # int phi_a' phi_b'
    s = [F(-1), F(1)]
    Cm = [[s[a] / 2 for _ in range(2)] for a in range(2)]  # int phi_a' phi_b
    return M, D, Cm


def grad_grad(h3, a, b, c, d):
    """int dN_a/dx_c * dN_b/dx_d over the brick."""
    out = F(1)
    for e in range(3):
        M, D, Cm = one_d(h3[e])
        ia, ib = NODES[a][e], NODES[b][e]
        if e == c and e == d:
            out *= D[ia][ib]
        elif e == c:
            out *= Cm[ia][ib]
        elif e == d:
            out *= Cm[ib][ia]
        else:
            out *= M[ia][ib]
    return out


def stiffness(h3, nu):
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1 / (2 * (1 + nu))
    K = [[F(0)] * 24 for _ in range(24)]
    for a in range(8):
        for b in range(8):
            for c in range(3):
                for d in range(3):
                    v = lam * grad_grad(h3, a, b, c, d) + mu * grad_grad(h3, a, b, d, c)
                    if c == d:
                        v += mu * sum(grad_grad(h3, a, b, e, e) for e in range(3))
                    K[3 * a + c][3 * b + d] = v
    return K


def scalar(h3):
    Ke = [[sum(grad_grad(h3, a, b, e, e) for e in range(3)) for b in range(8)] for a in range(8)]
    Me = [[F(1)] * 8 for _ in range(8)]
    for a in range(8):
        for b in range(8):
            v = F(1)
            for e in range(3):
                M, _, _ = one_d(h3[e])
                v *= M[NODES[a][e]][NODES[b][e]]
            Me[a][b] = v
    return Ke, Me


def flt(m):
    return [[float(x) for x in row] for row in m]


def main():
    cases = []
    for h3, nu in [((F(1), F(1), F(1)), F(3, 10)), ((F(1), F(2), F(1, 2)), F(3, 10)),
                   ((F(1), F(1), F(1)), F(1, 4)), ((F(3, 2), F(1), F(5, 4)), F(2, 5))]:
        K = stiffness(h3, nu)
        cases.append({"dx": float(h3[0]), "dy": float(h3[1]), "dz": float(h3[2]), "nu": float(nu),
                      "K0": flt(K), "K0_11_exact": f"{K[0][0].numerator}/{K[0][0].denominator}"})
    helm = []
    for h3, quirk in [((F(1), F(1), F(1)), True), ((F(1), F(1), F(1)), False), ((F(1), F(2), F(1, 2)), True)]:
        hz = h3[2] * F(3, 2) if quirk else h3[2]
        Ke, Me = scalar((h3[0], h3[1], hz))
        helm.append({"dx": float(h3[0]), "dy": float(h3[1]), "dz": float(h3[2]), "quirk": quirk,
                     "Ke": flt(Ke), "Me": flt(Me)})
    out = {"generator": "tests/golden/make_golden.py", "stiffness": cases, "helmholtz": helm}
    path = Path(__file__).with_name("element_kat.json")
    path.write_text(json.dumps(out, indent=1))
    print(path)


if __name__ == "__main__":
    main()
