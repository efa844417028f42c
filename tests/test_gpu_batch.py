"""Batches of uneven grids (hexa_solve_batch, hexa_filter_batch) against the
single-grid entry points and the oracle: each instance of a batch must give
what its own solve or filter gives."""
import ctypes as C

import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads
from v119_2025_12_19_hexatop_aws_gb300.helmholtz import filter_batch, filter_density
from v119_2025_12_19_hexatop_aws_gb300.solver import solve, solve_batch

pytestmark = pytest.mark.gpu

DIMS = [(16, 8, 8), (24, 12, 12), (8, 4, 4), (32, 16, 16), (12, 6, 6), (6, 3, 3), (48, 24, 24)]


def instances(rng, dims=DIMS, void=True):
    grids, facs, forces = [], [], []
    for q, d in enumerate(dims):
        ne = d[0] * d[1] * d[2]
        rho = np.clip(0.3 + 0.4 * rng.standard_normal(ne), 0.001, 1.0) if void else rng.uniform(0.1, 1.0, ne)
        facs.append(1e-9 + rho ** 3 * (1 - 1e-9))
        forces.append(workloads.point_loads(*d, 1, seed=100 + q)[0])
        grids.append(_lib.make_grid(*d))
    return grids, facs, forces


def test_batch_matches_single_solves(ctx, rng):
    grids, facs, forces = instances(rng)
    p = _lib.default_params(precision="mixed", divergence_check=0)
    U, stats, rc = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    assert rc == _lib.HEXA_OK
    p64 = _lib.default_params(precision="fp64", divergence_check=0, tol=1e-12)
    for i, g in enumerate(grids):
        assert stats[i]["status"] == 0 and stats[i]["true_relres"] <= 1e-9, i
        u, s = solve(g, facs[i], forces[i], clamp_faces=1, params=p64, ctx=ctx)
        assert np.linalg.norm(U[i] - u) <= 1e-7 * np.linalg.norm(u), i
        assert abs(stats[i]["compliance"] - s["compliance"]) <= 1e-8 * abs(s["compliance"]), i


def test_batch_matches_direct_solution(ctx, oracle, rng):
    dims = [(8, 4, 4), (12, 6, 6), (10, 4, 6)]
    grids, facs, forces = instances(rng, dims, void=False)
    p = _lib.default_params(precision="mixed", tol=1e-12, shift_factor=1e-10, divergence_check=0)
    U, stats, rc = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    assert rc == _lib.HEXA_OK
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    for i, d in enumerate(dims):
        g = oracle.Grid(*d)
        fixed = oracle.fixed_mask(g, 1)
        sigma = 1e-10 * oracle.diag_K(g, K0, facs[i], quirk=True)[~fixed].max()
        u_ref = oracle.direct_solve(g, K0, facs[i], forces[i], fixed, sigma)
        assert np.linalg.norm(U[i] - u_ref) <= 1e-9 * np.linalg.norm(u_ref), i


@pytest.mark.parametrize("faces,levels", [(1, [2, 2, 2, 2]), (1 | 2, [2, 2, 1, 1])])
def test_batch_odd_axes_coarsen_rounded_up(ctx, rng, faces, levels):
    """Odd axes keep coarsening (rounded up, the extra half element void)
    unless that axis' high face is clamped; either way each instance matches
    its own FP64 solve."""
    dims = [(22, 11, 11), (18, 9, 9), (15, 7, 9), (13, 9, 7)]
    grids, facs, forces = instances(rng, dims)
    # 1e-12: with E_min = 1e-9 voids a 1e-9 residual leaves u errors near 1e-6
    p = _lib.default_params(precision="mixed", tol=1e-12, divergence_check=0)
    U, stats, rc = solve_batch(grids, facs, forces, clamp_faces=faces, params=p, ctx=ctx)
    assert rc == _lib.HEXA_OK
    assert [s["mg_levels"] for s in stats] == levels
    p64 = _lib.default_params(precision="fp64", divergence_check=0, tol=1e-12)
    for i, g in enumerate(grids):
        assert stats[i]["status"] == 0 and stats[i]["true_relres"] <= 1e-12, i
        u, s = solve(g, facs[i], forces[i], clamp_faces=faces, params=p64, ctx=ctx)
        assert np.linalg.norm(U[i] - u) <= 1e-7 * np.linalg.norm(u), i


@pytest.mark.parametrize("dims", [[(12, 6, 6), (8, 4, 4)],      # scratch form (element products in shared memory)
                                  [(22, 11, 11), (8, 4, 4)],    # colour form (scratch does not fit)
                                  [(24, 12, 12), (8, 4, 4)]])   # global-memory form (vectors do not fit)
def test_batch_coarse_solve_forms(ctx, rng, dims):
    """One level: the preconditioner is the one-CTA coarse PCG alone, in the
    form the largest instance of the launch fits."""
    grids, facs, forces = instances(rng, dims, void=False)
    p = _lib.default_params(precision="mixed", tol=1e-11, divergence_check=0, mg_levels=1, max_iter=5000)
    U, stats, rc = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    assert rc == _lib.HEXA_OK
    p64 = _lib.default_params(precision="fp64", divergence_check=0, tol=1e-12)
    for i, g in enumerate(grids):
        assert stats[i]["status"] == 0 and stats[i]["mg_levels"] == 1, i
        u, s = solve(g, facs[i], forces[i], clamp_faces=1, params=p64, ctx=ctx)
        assert np.linalg.norm(U[i] - u) <= 1e-8 * np.linalg.norm(u), i


def test_batch_zero_load_instance_and_determinism(ctx, rng):
    grids, facs, forces = instances(rng, DIMS[:4])
    forces[2] = np.zeros_like(forces[2])
    p = _lib.default_params(precision="mixed", divergence_check=0)
    U1, s1, rc1 = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    U2, s2, rc2 = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    assert rc1 == rc2 == _lib.HEXA_OK
    assert not U1[2].any()
    assert all(np.array_equal(a, b) for a, b in zip(U1, U2))
    p.use_graphs = 0
    U3, s3, _ = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    assert all(np.array_equal(a, b) for a, b in zip(U1, U3))


def test_batch_autotune_caches_brick_depth(ctx, rng):
    grids, facs, forces = instances(rng, DIMS[:3])
    p = _lib.default_params(precision="mixed", divergence_check=0, autotune=1)
    U1, s1, _ = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    U2, s2, _ = solve_batch(grids, facs, forces, clamp_faces=1, params=p, ctx=ctx)
    assert all(s["true_relres"] <= 1e-9 for s in s1)
    assert all(np.array_equal(a, b) for a, b in zip(U1, U2))


def test_batch_rejects_unsupported_inputs(ctx, rng):
    grids, facs, forces = instances(rng, DIMS[:2])
    lib, n = ctx.lib, 2
    G = (_lib.Grid * n)(*grids)
    fp = (C.c_void_p * n)(*[_lib.ptr(a) for a in facs])
    ff = (C.c_void_p * n)(*[_lib.ptr(a) for a in forces])
    out = [np.empty_like(f) for f in forces]
    up = (C.c_void_p * n)(*[_lib.ptr(a) for a in out])
    mask = np.zeros(forces[0].size, dtype=np.uint8)
    bcs = (_lib.BC * n)(_lib.make_bc(1, mask), _lib.make_bc(1))
    p = _lib.default_params(precision="mixed")
    assert lib.hexa_solve_batch(ctx.h, n, G, bcs, 0.3, fp, ff, C.byref(p), up, None) == _lib.HEXA_ERR_ARG
    bcs = (_lib.BC * n)(_lib.make_bc(1), _lib.make_bc(1))
    pj = _lib.default_params(precision="mixed", precond="jacobi")
    assert lib.hexa_solve_batch(ctx.h, n, G, bcs, 0.3, fp, ff, C.byref(pj), up, None) == _lib.HEXA_ERR_ARG
    G2 = (_lib.Grid * n)(grids[0], _lib.make_grid(*DIMS[1], dx=2.0))
    assert lib.hexa_solve_batch(ctx.h, n, G2, bcs, 0.3, fp, ff, C.byref(p), up, None) == _lib.HEXA_ERR_ARG


@pytest.mark.parametrize("precision,bar", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_filter_batch_matches_single_filter(ctx, rng, precision, bar):
    dims = [(16, 8, 8), (24, 12, 12), (8, 4, 4), (40, 20, 20)]
    grids = [_lib.make_grid(*d) for d in dims]
    rhos = [rng.uniform(0.0, 1.0, d[0] * d[1] * d[2]) for d in dims]
    rhos[2] = np.zeros_like(rhos[2])  # a zero field comes back unchanged
    out, st = filter_batch(grids, rhos, 1.5, tol=1e-9, max_iter=2000, precision=precision, ctx=ctx)
    for i, g in enumerate(grids):
        ref, rs = filter_density(g, rhos[i], 1.5, tol=1e-9, max_iter=2000, precision=precision, ctx=ctx)
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(out[i] - ref).max() <= bar * scale, i
        assert abs(st[i]["iterations"] - rs["iterations"]) <= 10, i
