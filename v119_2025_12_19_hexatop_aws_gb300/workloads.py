"""Seeded synthetic cantilever workloads (no dataset is involved).

All grids are unit-cube hex8 elements, the x = 0 face fully clamped
(reference config ``location: [0, ':', ':'], DoFs: [1,2,3]``), E0 = 1,
Emin = 1e-9, nu = 0.3, penal = 3.

  c1  48x24x24, rho = 0.3 + U(-0.05, 0.05); total load -1 in z spread over the
      nodes of the bottom edge x = max, z = 0 (``location: ['100%', ':', 0]``,
      src/Core/Boundary.jl:280); SIMP + OC, Helmholtz radius 1.5 elements.
  c2  256x128x128, same BCs/load; rho = clamp(0.3 + 0.25 g, 0.001, 1) with g a
      seeded N(0,1) element field smoothed by the Helmholtz filter (radius 4
      elements), standardised, then renormalised to mean 0.3.
  c3  the c2 generator at 384x192x192.
  c4  the c2 grid and density, k = 8 unit point loads at seeded nodes of the
      x = max face with seeded unit directions.
  c5  64 instances, nx drawn from {16, 24, ..., 96}, ny = nz = nx/2, own
      density (radius 2) and own seeded point load.

Filter radii in elements r map to the Helmholtz length with the reference's
convention R = r*dx / 2.5 (src/Optimization/TopOpt.jl:300).
"""
from __future__ import annotations

import numpy as np

SEED = 20251219
E0, EMIN, NU, PENAL, VOLFRAC = 1.0, 1e-9, 0.3, 3.0, 0.3

SIZES = {"c1": (48, 24, 24), "c2": (256, 128, 128), "c3": (384, 192, 192), "c4": (256, 128, 128)}
MG_LEVELS = {"c2": 4, "c3": 5, "c4": 4}


def ndof(nx, ny, nz):
    return 3 * (nx + 1) * (ny + 1) * (nz + 1)


def edge_load(nx, ny, nz, total=-1.0):
    """Unit load in -z spread evenly over the nodes (nx, j, 0), j = 0..ny."""
    f = np.zeros(ndof(nx, ny, nz))
    NX = nx + 1
    nodes = nx + NX * np.arange(ny + 1)
    f[3 * nodes + 2] = total / (ny + 1)
    return f


def c1_density(nx=48, ny=24, nz=24, seed=SEED):
    rng = np.random.default_rng(seed)
    return 0.3 + rng.uniform(-0.05, 0.05, nx * ny * nz)


def helmholtz_R(r_elems: float, dx: float = 1.0) -> float:
    return r_elems * dx / 2.5


def smooth_density(nx, ny, nz, filter_fn, seed=SEED, r_elems=4.0, mean=0.3, lo=0.001, hi=1.0):
    """The c2/c3 generator.  filter_fn(g, R) -> filtered element field."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal(nx * ny * nz)
    gs = np.asarray(filter_fn(g, helmholtz_R(r_elems)), dtype=np.float64)
    gs = (gs - gs.mean()) / gs.std()
    rho = np.clip(mean + 0.25 * gs, lo, hi)
    for _ in range(200):
        m = rho.mean()
        if abs(m - mean) < 1e-12:
            break
        rho = np.clip(rho + (mean - m), lo, hi)
    return rho


def point_loads(nx, ny, nz, k, seed=SEED):
    """k unit point loads at seeded nodes of the x = max face, seeded unit directions."""
    rng = np.random.default_rng(seed + 4)
    F = np.zeros((k, ndof(nx, ny, nz)))
    NX, NY = nx + 1, ny + 1
    for q in range(k):
        j = int(rng.integers(0, ny + 1))
        kk = int(rng.integers(0, nz + 1))
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        n = nx + NX * (j + NY * kk)
        F[q, 3 * n:3 * n + 3] = d
    return F


def batch_sizes(n=64, seed=SEED):
    rng = np.random.default_rng(seed + 5)
    nxs = rng.choice(np.arange(16, 97, 8), size=n)
    return [(int(x), int(x) // 2, int(x) // 2) for x in nxs]
