"""(a)-(c) GPU solves through the C ABI against the oracle: direct LU
solutions of the same shifted system, and the reference's Jacobi-PCG control
flow restated (GPUSolver.jl:182-465)."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads
from v119_2025_12_19_hexatop_aws_gb300.boundary import apply_external_forces, get_bc_indicator
from v119_2025_12_19_hexatop_aws_gb300.mesh import generate_mesh
from v119_2025_12_19_hexatop_aws_gb300.solver import solve, solve_system, solve_system_gpu

pytestmark = pytest.mark.gpu


def cantilever(oracle, rng, dims, lo=0.1, hi=1.0):
    g = oracle.Grid(*dims)
    fac = rng.uniform(lo, hi, g.nelem)
    f = workloads.edge_load(*dims)
    fixed = oracle.fixed_mask(g, 1)
    return g, fac, f, fixed


def shift_of(oracle, g, fac, fixed, factor=1e-10):
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    return factor * oracle.diag_K(g, K0, fac, quirk=True)[~fixed].max()


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("precond", ["jacobi", "multigrid"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("shift_factor", [0.0, 1e-10])
def test_solution_matches_direct(ctx, oracle, rng, precond, precision, shift_factor):
    """Both systems against LU: the unshifted K_ff u = f (shift_factor 0) and
    the reference's shifted (K_ff + sigma I) u = f, sigma = 1e-10 max diag
    (GPUSolver.jl:343).  unshifted_relres is ||f - K u|| / ||f|| in FP64."""
    dims = (16, 8, 8)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    sigma = shift_of(oracle, g, fac, fixed, factor=shift_factor)
    u_ref = oracle.direct_solve(g, K0, fac, f, fixed, sigma)
    p = _lib.default_params(precond=precond, precision=precision, tol=1e-13, max_iter=20000, mg_levels=3,
                            shift_factor=shift_factor)
    u, st = solve(_lib.make_grid(*dims), fac, f, clamp_faces=1, params=p, ctx=ctx)
    assert st["status"] == 0
    assert st["shift"] == pytest.approx(sigma, rel=1e-12, abs=0.0)
    assert st["true_relres"] <= 1e-13
    r_unshifted = np.linalg.norm(f * ~fixed - oracle.apply_A(g, K0, fac, u, fixed)) / np.linalg.norm(f)
    # at a 1e-13 residual the FP64 recomputations (GPU and oracle) differ in their own rounding
    assert abs(st["unshifted_relres"] - r_unshifted) <= 0.1 * r_unshifted + 1e-14
    if shift_factor == 0.0:
        assert st["unshifted_relres"] == st["true_relres"]
    assert rel(u, u_ref) <= 1e-10
    assert abs(f @ u - f @ u_ref) <= 1e-10 * abs(f @ u_ref)
    assert st["compliance"] == pytest.approx(f @ u_ref, rel=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_unshifted_void_contrast_reaches_fp64_residual(ctx, oracle, rng, precision):
    """SIMP factors down to 1e-9 (void contrast): with shift_factor 0 the solve
    reaches ||f - K u|| / ||f|| <= 1e-9 and matches LU of the unshifted system;
    with the reference's shift the same solve leaves the unshifted residual at
    about sigma ||u|| / ||f||."""
    dims = (24, 12, 12)
    g = oracle.Grid(*dims)
    rho = np.clip(0.3 + 0.35 * rng.standard_normal(g.nelem), 1e-3, 1.0)
    fac = 1e-9 + rho ** 3 * (1 - 1e-9)
    f = workloads.edge_load(*dims)
    fixed = oracle.fixed_mask(g, 1)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    u_ref = oracle.direct_solve(g, K0, fac, f, fixed, 0.0)
    grid = _lib.make_grid(*dims)
    p = _lib.default_params(precision=precision, tol=1e-9, max_iter=60000, divergence_check=0, shift_factor=0.0)
    u, st = solve(grid, fac, f, clamp_faces=1, params=p, ctx=ctx)
    assert st["status"] == 0 and st["shift"] == 0.0
    assert st["unshifted_relres"] <= 1e-9
    r = np.linalg.norm(f * ~fixed - oracle.apply_A(g, K0, fac, u, fixed)) / np.linalg.norm(f)
    assert r <= 1.05e-9
    assert abs(f @ u - f @ u_ref) <= 1e-10 * abs(f @ u_ref)
    ps = _lib.default_params(precision=precision, tol=1e-9, max_iter=60000, divergence_check=0, shift_factor=1e-10)
    us, sts = solve(grid, fac, f, clamp_faces=1, params=ps, ctx=ctx)
    assert sts["true_relres"] <= 1e-9
    expect = sts["shift"] * np.linalg.norm(us) / np.linalg.norm(f)
    assert sts["unshifted_relres"] == pytest.approx(expect, rel=0.5)


def test_fp32_solution_close(ctx, oracle, rng):
    dims = (16, 8, 8)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    u_ref = oracle.direct_solve(g, K0, fac, f, fixed, shift_of(oracle, g, fac, fixed))
    p = _lib.default_params(precond="jacobi", precision="fp32", tol=1e-5, max_iter=20000)
    u, st = solve(_lib.make_grid(*dims), fac, f, clamp_faces=1, params=p, ctx=ctx)
    assert rel(u, u_ref) <= 1e-3


@pytest.mark.parametrize("dims", [(12, 6, 6), (20, 10, 10)])
def test_jacobi_iteration_count_matches_reference(ctx, oracle, rng, dims):
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    u_ref, rel_ref, info = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-9, max_iter=20000, shift_factor=1e-10)
    p = _lib.default_params(precond="jacobi", tol=1e-9, max_iter=20000, check_cadence=10, true_residual=0)
    u, st = solve(_lib.make_grid(*dims), fac, f, clamp_faces=1, params=p, ctx=ctx)
    assert st["status"] == 0 and info.success
    assert abs(st["iterations"] - info.iterations[-1]) <= 10
    assert st["relres"] < 1e-9
    assert rel(u, u_ref) < 1e-7


def test_multigrid_beats_jacobi(ctx, oracle, rng):
    dims = (32, 16, 16)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    grid = _lib.make_grid(*dims)
    _, sj = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(precond="jacobi"), ctx=ctx)
    _, sm = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(precond="multigrid"), ctx=ctx)
    assert sm["status"] == 0 and sj["status"] == 0
    assert sm["iterations"] * 3 < sj["iterations"]
    assert sm["true_relres"] <= 1e-9 and sj["true_relres"] <= 1e-9


def test_solve_is_deterministic(ctx, oracle, rng):
    dims = (24, 12, 12)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    grid = _lib.make_grid(*dims)
    u1, _ = solve(grid, fac, f, clamp_faces=1, ctx=ctx)
    u2, _ = solve(grid, fac, f, clamp_faces=1, ctx=ctx)
    assert np.array_equal(u1, u2)


def test_without_graphs_same_answer(ctx, oracle, rng):
    dims = (16, 8, 8)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    grid = _lib.make_grid(*dims)
    u1, s1 = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(use_graphs=1), ctx=ctx)
    u2, s2 = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(use_graphs=0), ctx=ctx)
    assert np.array_equal(u1, u2) and s1["iterations"] == s2["iterations"]


def _reference_inputs(dims):
    nodes, elements, _ = generate_mesh(*dims)
    bc = get_bc_indicator(nodes.shape[0], nodes, [{"location": [0, ":", ":"], "DoFs": [1, 2, 3]}])
    F = np.zeros(3 * nodes.shape[0], dtype=np.float32)
    apply_external_forces(F, [{"location": ["100%", ":", 0], "F": [0, 0, -1]}], nodes)
    return nodes, elements, bc, F


def test_reference_signature_entry_point(ctx, oracle, rng):
    dims = (12, 6, 6)
    nodes, elements, bc, F = _reference_inputs(dims)
    dens = rng.uniform(0.2, 1.0, 12 * 6 * 6).astype(np.float32)
    cfg = {"solver_parameters": {"preconditioner": "multigrid", "max_shift_attempts": 5, "shift_multiplier": 4.0},
           "hardware_profile_applied": "H100", "force_float64": True, "geometry": {}}
    u, relres, name = solve_system_gpu(nodes, elements, np.float32(1.0), np.float32(0.3), bc, F, dens, tol=1e-9,
                                       max_iter=30000, shift_factor=1e-10, config=cfg)
    assert name == "GMG_GPU" and relres < 1e-9
    g = oracle.Grid(*dims)
    fixed = oracle.fixed_mask(g, 0, (bc > 0).astype(np.uint8).ravel())
    fac = (np.float32(1.0) * dens).astype(np.float64)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    sigma = 1e-10 * oracle.diag_K(g, K0, fac, quirk=True)[~fixed].max()
    u_ref = oracle.direct_solve(g, K0, fac, F.astype(np.float64), fixed, sigma)
    assert rel(u, u_ref) < 1e-7
    assert np.all(u[fixed] == 0)


def test_solve_system_dispatch(ctx, rng):
    dims = (8, 4, 4)
    nodes, elements, bc, F = _reference_inputs(dims)
    dens = np.full(8 * 4 * 4, 0.5, dtype=np.float32)
    cfg = {"solver_parameters": {"solver_type": "gpu", "preconditioner": "jacobi", "tolerance": 1e-9,
                                 "max_iterations": 30000, "diagonal_shift_factor": 1e-10}, "force_float64": True,
           "geometry": {}}
    u, relres, name = solve_system(nodes, elements, 1.0, 0.3, bc, F, density=dens, config=cfg, prune_voids=False)
    assert name == "Jacobi_GPU" and relres < 1e-9


def test_corrupt_input_returns_sentinel(ctx):
    dims = (6, 3, 3)
    nodes, elements, bc, F = _reference_inputs(dims)
    dens = np.full(6 * 3 * 3, 0.5, dtype=np.float32)
    dens[5] = np.nan
    u, relres, name = solve_system_gpu(nodes, elements, 1.0, 0.3, bc, F, dens, tol=1e-9, config={"force_float64": True})
    assert name == "Failed_Corrupt_Input" and np.isnan(relres) and not u.any()


def test_max_iter_returns_best_iterate_not_converged(ctx, oracle, rng):
    dims = (16, 8, 8)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    p = _lib.default_params(precond="jacobi", max_iter=5, max_shift_attempts=1)
    u, st = solve(_lib.make_grid(*dims), fac, f, clamp_faces=1, params=p, ctx=ctx)
    assert st["status"] == _lib.HEXA_NOT_CONVERGED
    assert np.isfinite(u).all() and np.abs(u).max() > 0


def test_u_guess_warm_start(ctx, oracle, rng):
    dims = (16, 8, 8)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    grid = _lib.make_grid(*dims)
    p = _lib.default_params(precond="jacobi")
    u, s0 = solve(grid, fac, f, clamp_faces=1, params=p, ctx=ctx)
    u2, s1 = solve(grid, fac, f, clamp_faces=1, params=p, u_guess=u, ctx=ctx)
    assert s1["iterations"] < s0["iterations"] // 4


def test_zero_load_gives_zero(ctx, oracle, rng):
    dims = (6, 3, 3)
    g, fac, f, fixed = cantilever(oracle, rng, dims)
    u, st = solve(_lib.make_grid(*dims), fac, np.zeros_like(f), clamp_faces=1, ctx=ctx)
    assert st["status"] == 0 and not u.any()


def test_void_contrast_mixed_reaches_fp64_residual(ctx, oracle, rng):
    dims = (32, 16, 16)
    g = oracle.Grid(*dims)
    rho = np.clip(0.3 + 0.4 * rng.standard_normal(g.nelem), 0.001, 1.0)
    fac = 1e-9 + rho ** 3 * (1 - 1e-9)
    f = workloads.edge_load(*dims)
    grid = _lib.make_grid(*dims)
    u64, s64 = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(precision="fp64"), ctx=ctx)
    um, sm = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(precision="mixed"), ctx=ctx)
    assert s64["true_relres"] <= 1e-9 and sm["true_relres"] <= 1e-9
    assert abs(sm["compliance"] - s64["compliance"]) <= 1e-8 * abs(s64["compliance"])


def test_autotuned_mixed_matches_fp64_and_caches(ctx, oracle, rng):
    dims = (32, 16, 16)
    g = oracle.Grid(*dims)
    rho = np.clip(0.3 + 0.3 * rng.standard_normal(g.nelem), 0.001, 1.0)
    fac = 1e-9 + rho ** 3 * (1 - 1e-9)
    f = workloads.edge_load(*dims)
    grid = _lib.make_grid(*dims)
    u64, s64 = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(divergence_check=0), ctx=ctx)
    p = _lib.default_params(precision="mixed", autotune=1, divergence_check=0)
    um, s1 = solve(grid, fac, f, clamp_faces=1, params=p, ctx=ctx)
    um2, s2 = solve(grid, fac, f, clamp_faces=1, params=p, ctx=ctx)
    assert s1["status"] == 0 and s1["true_relres"] <= 1e-9
    assert s1["smooth_steps"] in (2, 3, 4, 5) and s1["mg_levels"] >= 2
    assert (s2["mg_levels"], s2["smooth_steps"]) == (s1["mg_levels"], s1["smooth_steps"])
    assert s2["setup_ms"] < s1["setup_ms"]  # the second call reuses the tuned settings
    assert np.array_equal(um, um2)
    assert abs(s1["compliance"] - s64["compliance"]) <= 1e-8 * abs(s64["compliance"])


def test_mixed_matches_fp64_on_a_grid_with_interior_tiles(ctx, oracle, rng):
    """64x32x16: the FP32 smoothing, residual and PCG operator forms run both
    their interior-tile and boundary-tile item paths."""
    dims = (64, 32, 16)
    g = oracle.Grid(*dims)
    rho = np.clip(0.3 + 0.3 * rng.standard_normal(g.nelem), 0.001, 1.0)
    fac = 1e-9 + rho ** 3 * (1 - 1e-9)
    f = workloads.edge_load(*dims)
    grid = _lib.make_grid(*dims)
    u64, s64 = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(divergence_check=0, tol=1e-11), ctx=ctx)
    um, sm = solve(grid, fac, f, clamp_faces=1, params=_lib.default_params(precision="mixed", divergence_check=0,
                                                                           tol=1e-11), ctx=ctx)
    assert s64["status"] == 0 and sm["status"] == 0
    assert sm["true_relres"] <= 1e-11
    assert np.linalg.norm(um - u64) <= 1e-7 * np.linalg.norm(u64)
    assert abs(sm["compliance"] - s64["compliance"]) <= 1e-10 * abs(s64["compliance"])


def _voided_density(oracle, g, seed, void_frac=0.15, thr=1e-3):
    rng = np.random.default_rng(seed)
    s = oracle.helmholtz_direct(g, rng.standard_normal(g.nelem), 0.8, quirk=False)
    rho = np.clip(0.3 + 0.4 * (s - s.mean()) / s.std(), 0.05, 1.0)
    rho[s <= np.quantile(s, void_frac)] = thr
    return rho.astype(np.float32)


@pytest.mark.parametrize("shift_factor", [1e-10, 0.0])
def test_solve_system_prunes_voids_like_the_reference(ctx, oracle, shift_factor):
    """Main.jl:439-443 calls Solver.solve_system with prune_voids=true.  From
    outer iteration 3, with 15 % of the elements at the minimum density, the
    reference solves MeshPruner's compacted system and maps it back
    (Solver.jl:85-156); the oracle restates exactly that (renumbered mesh,
    assembled, Jacobi-PCG to 1e-14).  The library's solve_system on the full
    structured mesh gives the same U_full within 1e-10, zeros at the removed
    nodes, and the unpruned solve before iteration 3."""
    dims = workloads.SIZES["c1"]
    g = oracle.Grid(*dims)
    nodes, elements, bc, F = _reference_inputs(dims)
    dens = _voided_density(oracle, g, seed=11)
    cfg = {"solver_parameters": {"solver_type": "gpu", "preconditioner": "multigrid", "tolerance": 1e-13,
                                 "max_iterations": 60000, "diagonal_shift_factor": shift_factor},
           "force_float64": True, "geometry": {}, "current_outer_iter": 3}
    st = {}
    u, relres, name = solve_system(nodes, elements, 1.0, 0.3, bc, F, density=dens, config=cfg,
                                   min_stiffness_threshold=np.float32(1e-3), prune_voids=True, stats=st)
    assert name == "GMG_GPU" and st["status"] == 0
    u_ref, nact = oracle.solve_system_pruned(g, 1.0, dens, bc, F, min_stiffness_threshold=np.float32(1e-3),
                                             prune_voids=True, current_outer_iter=3, shift_factor=float(np.float32(shift_factor)))
    assert st["active_elements"] == nact < 0.99 * g.nelem
    assert rel(u, u_ref) <= 1e-10
    assert abs(F @ u - F @ u_ref) <= 1e-10 * abs(F @ u_ref)
    on = np.zeros(g.nnode, dtype=bool)
    on[oracle.element_nodes(g)[dens > np.float32(1e-3) * np.float32(1.01)].ravel()] = True
    assert (~on).any() and not u.reshape(-1, 3)[~on].any()  # reconstruct_full_solution's zeros
    cfg2 = dict(cfg, current_outer_iter=2)
    st2 = {}
    solve_system(nodes, elements, 1.0, 0.3, bc, F, density=dens, config=cfg2, min_stiffness_threshold=np.float32(1e-3),
                 prune_voids=True, stats=st2)
    assert st2["active_elements"] == g.nelem


def test_solve_system_with_every_element_pruned_is_an_error(ctx):
    dims = (8, 4, 4)
    nodes, elements, bc, F = _reference_inputs(dims)
    cfg = {"solver_parameters": {"solver_type": "gpu", "tolerance": 1e-9, "diagonal_shift_factor": 1e-10},
           "force_float64": True, "geometry": {}, "current_outer_iter": 5}
    with pytest.raises(_lib.HexaError, match="No active elements"):
        solve_system(nodes, elements, 1.0, 0.3, bc, F, density=np.full(128, 1e-3, np.float32), config=cfg,
                     min_stiffness_threshold=np.float32(1e-3), prune_voids=True)
