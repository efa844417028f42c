"""Void pruning of Solver.solve_system (src/Solvers/Solver.jl:66-104,
src/Mesh/MeshPruner.jl:10-107) in the oracle, on CPU: the restated pruner
renumbers as the reference does, and the pruned unstructured system it builds
has the same solution as the structured grid with the pruned elements'
factors set to zero and the removed nodes fixed -- the form the library
solves."""
import numpy as np
import pytest


def voided_density(oracle, g, seed, void_frac=0.15, thr=1e-3):
    """A smooth seeded field with its lowest `void_frac` of elements at the
    minimum density `thr` (connected void regions, as culling leaves them)."""
    rng = np.random.default_rng(seed)
    s = oracle.helmholtz_direct(g, rng.standard_normal(g.nelem), 0.8, quirk=False)
    rho = np.clip(0.3 + 0.4 * (s - s.mean()) / s.std(), 0.05, 1.0)
    rho[s <= np.quantile(s, void_frac)] = thr
    return rho.astype(np.float32)


def test_prune_system_renumbers_like_meshpruner(oracle):
    g = oracle.Grid(3, 2, 1)
    el = oracle.element_nodes(g)
    dens = np.array([1, 0.001, 0.001, 0.001, 0.001, 1], dtype=np.float32)
    nodes = np.arange(3 * g.nnode, dtype=np.float32).reshape(-1, 3)
    bc = np.zeros((g.nnode, 3), dtype=np.float32)
    bc[0] = 1
    F = np.arange(3 * g.nnode, dtype=np.float32)
    P = oracle.prune_system(nodes, el, dens, np.float32(1e-3) * np.float32(1.01), bc, F)
    keep = np.unique(el[[0, 5]].ravel())
    assert np.array_equal(P["new_to_old_node_map"], keep)
    assert np.array_equal(P["active_element_indices"], [0, 5])
    assert P["elements"].max() == keep.size - 1
    assert np.array_equal(keep[P["elements"]], el[[0, 5]])
    assert np.array_equal(P["F"], F.reshape(-1, 3)[keep].ravel())
    assert np.array_equal(P["bc_indicator"], bc[keep])
    u = oracle.reconstruct_full_solution(np.ones(3 * keep.size), keep, g.nnode).reshape(-1, 3)
    assert u[keep].all() and not np.delete(u, keep, axis=0).any()
    with pytest.raises(ValueError, match="No active elements"):
        oracle.prune_system(nodes, el, np.full(6, 1e-3, np.float32), 1.0, bc, F)


@pytest.mark.parametrize("shift_factor", [0.0, 1e-10])
def test_pruned_system_equals_zero_factor_form(oracle, shift_factor):
    """The pruned system, assembled on its own renumbered mesh and mapped back,
    equals the structured system with zero factors on pruned elements and the
    removed nodes' DOFs fixed (same shift from the same diagonal)."""
    g = oracle.Grid(10, 5, 5)
    dens = voided_density(oracle, g, seed=3)
    bc = np.zeros((g.nnode, 3), dtype=np.float32)
    bc[oracle.fixed_mask(g, 1).reshape(-1, 3).all(axis=1)] = 1.0
    from v119_2025_12_19_hexatop_aws_gb300 import workloads
    F = workloads.edge_load(10, 5, 5).astype(np.float32)
    u_p, nact = oracle.solve_system_pruned(g, 1.0, dens, bc, F, min_stiffness_threshold=1e-3, prune_voids=True,
                                           current_outer_iter=3, shift_factor=shift_factor)
    thr = np.float32(1e-3) * np.float32(1.01)
    act = dens > thr
    assert nact == act.sum() < 0.99 * g.nelem
    el = oracle.element_nodes(g)
    on = np.zeros(g.nnode, dtype=bool)
    on[el[act].ravel()] = True
    fixed = (bc.reshape(-1) > 0) | np.repeat(~on, 3)
    fac = np.where(act, dens, 0.0).astype(np.float64)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    sigma = shift_factor * oracle.diag_K(g, K0, fac, quirk=True)[~fixed].max()
    u_z = oracle.direct_solve(g, K0, fac, F.astype(np.float64) * ~fixed, fixed, sigma)
    assert np.linalg.norm(u_p - u_z) <= 1e-10 * np.linalg.norm(u_z)
    assert not u_p.reshape(-1, 3)[~on].any()


def test_no_pruning_before_iteration_3_or_above_99_percent(oracle):
    g = oracle.Grid(6, 3, 3)
    dens = voided_density(oracle, g, seed=4)
    bc = np.zeros((g.nnode, 3), dtype=np.float32)
    bc[oracle.fixed_mask(g, 1).reshape(-1, 3).all(axis=1)] = 1.0
    from v119_2025_12_19_hexatop_aws_gb300 import workloads
    F = workloads.edge_load(6, 3, 3).astype(np.float32)
    kw = dict(min_stiffness_threshold=1e-3, shift_factor=1e-10)
    _, n2 = oracle.solve_system_pruned(g, 1.0, dens, bc, F, prune_voids=True, current_outer_iter=2, **kw)
    _, n3 = oracle.solve_system_pruned(g, 1.0, dens, bc, F, prune_voids=True, current_outer_iter=3, **kw)
    _, nf = oracle.solve_system_pruned(g, 1.0, dens, bc, F, prune_voids=False, current_outer_iter=9, **kw)
    assert n2 == nf == g.nelem and n3 < g.nelem
    g2 = oracle.Grid(12, 6, 6)
    bc2 = np.zeros((g2.nnode, 3), dtype=np.float32)
    bc2[oracle.fixed_mask(g2, 1).reshape(-1, 3).all(axis=1)] = 1.0
    F2 = workloads.edge_load(12, 6, 6).astype(np.float32)
    few = np.full(g2.nelem, 0.5, dtype=np.float32)
    few[:4] = 1e-3  # 4 void elements in 432: above 99 % active, no pruning
    _, n = oracle.solve_system_pruned(g2, 1.0, few, bc2, F2, prune_voids=True, current_outer_iter=5, **kw)
    assert n == g2.nelem
    few[:5] = 1e-3  # 5 in 432: below 99 % active, pruned
    _, n = oracle.solve_system_pruned(g2, 1.0, few, bc2, F2, prune_voids=True, current_outer_iter=5, **kw)
    assert n == g2.nelem - 5
