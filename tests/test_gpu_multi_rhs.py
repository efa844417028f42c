"""k load cases as one block PCG (hexa_solve_multi_rhs) against the oracle.

Every column must match the direct solution of the same shifted system (the
oracle's LU), and the mixed form must reach the FP64 residual bar per column;
dependent and zero columns exercise the pseudo-inverse of the block step.
"""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads
from v119_2025_12_19_hexatop_aws_gb300.solver import solve, solve_multi_rhs

pytestmark = pytest.mark.gpu


def setup(oracle, rng, dims, k, void=False):
    g = oracle.Grid(*dims)
    if void:
        rho = np.clip(0.3 + 0.4 * rng.standard_normal(g.nelem), 0.001, 1.0)
        fac = 1e-9 + rho ** 3 * (1 - 1e-9)
    else:
        fac = rng.uniform(0.1, 1.0, g.nelem)
    F = workloads.point_loads(*dims, k)
    fixed = oracle.fixed_mask(g, 1)
    return g, fac, F, fixed


def direct(oracle, g, fac, F, fixed, shift_factor=1e-10):
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    sigma = shift_factor * oracle.diag_K(g, K0, fac, quirk=True)[~fixed].max()
    return np.stack([oracle.direct_solve(g, K0, fac, F[j], fixed, sigma) for j in range(F.shape[0])])


def colrel(U, R):
    return max(np.linalg.norm(U[j] - R[j]) / np.linalg.norm(R[j]) for j in range(R.shape[0]) if R[j].any())


@pytest.mark.parametrize("precond", ["jacobi", "multigrid"])
def test_block_fp64_matches_direct(ctx, oracle, rng, precond):
    dims = (16, 8, 8)
    g, fac, F, fixed = setup(oracle, rng, dims, 4)
    R = direct(oracle, g, fac, F, fixed)
    p = _lib.default_params(precond=precond, precision="fp64", tol=1e-12, max_iter=20000, mg_levels=3)
    U, st = solve_multi_rhs(_lib.make_grid(*dims), fac, F, clamp_faces=1, params=p, ctx=ctx)
    assert st["status"] == 0 and st["true_relres"] <= 1e-12
    assert colrel(U, R) <= 1e-10
    assert st["compliance"] == pytest.approx(sum(F[j] @ R[j] for j in range(4)), rel=1e-10)


def test_block_mixed_void_contrast_per_column(ctx, oracle, rng):
    dims = (32, 16, 16)
    g, fac, F, fixed = setup(oracle, rng, dims, 8, void=True)
    grid = _lib.make_grid(*dims)
    p = _lib.default_params(precision="mixed", divergence_check=0)
    U, st = solve_multi_rhs(grid, fac, F, clamp_faces=1, params=p, ctx=ctx)
    assert st["status"] == 0 and st["true_relres"] <= 1e-9
    # each column against its own FP64 single solve
    p64 = _lib.default_params(precision="fp64", divergence_check=0, tol=1e-12)
    total = 0.0
    for j in range(8):
        u, s = solve(grid, fac, F[j], clamp_faces=1, params=p64, ctx=ctx)
        assert np.linalg.norm(U[j] - u) <= 1e-7 * np.linalg.norm(u)
        total += s["compliance"]
    assert abs(st["compliance"] - total) <= 1e-8 * abs(total)


def test_block_handles_dependent_and_zero_columns(ctx, oracle, rng):
    dims = (16, 8, 8)
    g, fac, F0, fixed = setup(oracle, rng, dims, 3)
    F = np.stack([F0[0], 2.0 * F0[0], np.zeros_like(F0[0]), F0[1]])
    R = direct(oracle, g, fac, F, fixed)
    for precision, tol, bar in (("fp64", 1e-12, 1e-10), ("mixed", 1e-10, 1e-8)):
        p = _lib.default_params(precond="multigrid", precision=precision, tol=tol, max_iter=20000, mg_levels=3)
        U, st = solve_multi_rhs(_lib.make_grid(*dims), fac, F, clamp_faces=1, params=p, ctx=ctx)
        assert st["status"] == 0, precision
        assert not U[2].any()
        assert colrel(U, R) <= bar, precision


def test_block_single_column_and_groups_of_sixteen(ctx, oracle, rng):
    dims = (12, 6, 6)
    g, fac, F, fixed = setup(oracle, rng, dims, 17)
    R = direct(oracle, g, fac, F, fixed)
    p = _lib.default_params(precond="multigrid", precision="fp64", tol=1e-12, max_iter=20000, mg_levels=2)
    grid = _lib.make_grid(*dims)
    U, st = solve_multi_rhs(grid, fac, F, clamp_faces=1, params=p, ctx=ctx)  # 16 + 1 columns
    assert st["status"] == 0 and colrel(U, R) <= 1e-10
    U1, st1 = solve_multi_rhs(grid, fac, F[:1].copy(), clamp_faces=1, params=p, ctx=ctx)
    assert st1["status"] == 0 and colrel(U1, R[:1]) <= 1e-10


def test_block_is_deterministic_and_graphs_agree(ctx, oracle, rng):
    dims = (16, 8, 8)
    g, fac, F, fixed = setup(oracle, rng, dims, 8, void=True)
    grid = _lib.make_grid(*dims)
    p = _lib.default_params(precision="mixed", divergence_check=0)
    U1, s1 = solve_multi_rhs(grid, fac, F, clamp_faces=1, params=p, ctx=ctx)
    U2, s2 = solve_multi_rhs(grid, fac, F, clamp_faces=1, params=p, ctx=ctx)
    assert np.array_equal(U1, U2) and s1["iterations"] == s2["iterations"]
    p.use_graphs = 0
    U3, s3 = solve_multi_rhs(grid, fac, F, clamp_faces=1, params=p, ctx=ctx)
    assert np.array_equal(U1, U3)
