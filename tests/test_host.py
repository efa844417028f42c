"""Host-side logic: mesh numbering (Mesh.jl), BC/load input semantics
(Boundary.jl), config mapping, workload generators.  CPU only."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import workloads
from v119_2025_12_19_hexatop_aws_gb300.boundary import (apply_external_forces, bc_to_fixed_dof, face_clamps,
                                                        get_bc_indicator, nodes_by_location)
from v119_2025_12_19_hexatop_aws_gb300.mesh import generate_mesh, node_index, structured_dims
from v119_2025_12_19_hexatop_aws_gb300.solver import params_from_config, precision_from_config


def test_mesh_numbering_matches_mesh_jl():
    nodes, elems, dims = generate_mesh(3, 2, 2, 1.0, 2.0, 0.5)
    assert dims == (4, 3, 3) and nodes.dtype == np.float32
    # Mesh.jl:45-53 element 1 = nodes (1,1,1),(2,1,1),(2,2,1),(1,2,1),(1,1,2),...
    e = elems[0]
    assert list(e) == [node_index(1, 1, 1, 4, 3), node_index(2, 1, 1, 4, 3), node_index(2, 2, 1, 4, 3),
                       node_index(1, 2, 1, 4, 3), node_index(1, 1, 2, 4, 3), node_index(2, 1, 2, 4, 3),
                       node_index(2, 2, 2, 4, 3), node_index(1, 2, 2, 4, 3)]
    assert np.allclose(nodes[node_index(4, 3, 3, 4, 3) - 1], [3.0, 4.0, 1.0])
    assert elems.max() == nodes.shape[0]


def test_structured_dims_roundtrip_and_rejects_pruned():
    nodes, elems, _ = generate_mesh(5, 3, 4, 1.0, 2.0, 0.5)
    assert structured_dims(nodes, elems) == (5, 3, 4, 1.0, 2.0, 0.5)
    with pytest.raises(ValueError):
        structured_dims(nodes, elems[:-1])
    bad = elems.copy()
    bad[0, [0, 1]] = bad[0, [1, 0]]
    with pytest.raises(ValueError):
        structured_dims(nodes, bad)


def test_location_grammar():
    nodes, _, _ = generate_mesh(10, 4, 4, 1.0, 1.0, 1.0)
    x0 = nodes_by_location([0, ":", ":"], nodes)
    assert np.all(nodes[x0, 0] == 0) and x0.size == 25
    # a number in [0,1] is a FRACTION of the extent (Boundary.jl:119)
    half = nodes_by_location([0.5, ":", ":"], nodes)
    assert np.all(nodes[half, 0] == 5.0)
    # numbers outside [0,1] are coordinates
    three = nodes_by_location([3, ":", ":"], nodes)
    assert np.all(nodes[three, 0] == 3.0)
    edge = nodes_by_location(["100%", ":", 0], nodes)
    assert np.all(nodes[edge, 0] == 10) and np.all(nodes[edge, 2] == 0) and edge.size == 5
    with pytest.raises(ValueError):
        nodes_by_location([0, ":"], nodes)


def test_bc_indicator_and_forces():
    nodes, _, _ = generate_mesh(8, 4, 4)
    bc = get_bc_indicator(nodes.shape[0], nodes, [{"location": [0, ":", ":"], "DoFs": [1, 2, 3]},
                                                   {"node": 7, "DoFs": [2]}])
    assert bc.shape == (nodes.shape[0], 3) and bc[:, 0].sum() == 25 and bc[6, 1] == 1
    F = np.zeros(3 * nodes.shape[0], dtype=np.float32)
    apply_external_forces(F, [{"location": ["100%", ":", 0], "F": [0, 0, -1]}], nodes)
    assert F[2::3].sum() == pytest.approx(-1.0) and np.count_nonzero(F) == 5
    # point location with no exact match maps to the nearest node
    F2 = np.zeros_like(F)
    apply_external_forces(F2, [{"location": [8.0, 2.2, 3.9], "F": [1, 0, 0]}], nodes)
    n = np.nonzero(F2)[0]
    assert n.size == 1 and np.allclose(nodes[n[0] // 3], [8, 2, 4])
    with pytest.raises(ValueError):
        get_bc_indicator(nodes.shape[0], nodes, [{"location": [0, ":", ":"], "DoFs": [4]}])


def test_face_clamp_detection():
    nodes, elems, _ = generate_mesh(6, 3, 3)
    bc = get_bc_indicator(nodes.shape[0], nodes, [{"location": [0, ":", ":"], "DoFs": [1, 2, 3]}])
    faces, rest = face_clamps(bc_to_fixed_dof(bc), 6, 3, 3)
    assert faces == 1 and rest is None
    bc[10, 1] = 1
    faces, rest = face_clamps(bc_to_fixed_dof(bc), 6, 3, 3)
    assert faces == 1 and rest is not None and rest.sum() == 16 * 3 + 1


def test_precision_rules():
    assert precision_from_config({"hardware_profile_applied": "H200"}) == "fp64"
    assert precision_from_config({"hardware_profile_applied": "RTX"}) == "fp32"
    assert precision_from_config({"force_float64": True}) == "fp64"
    assert precision_from_config({"solver_parameters": {"precision": "mixed"}}) == "mixed"


def test_params_from_config(built_lib):
    cfg = {"solver_parameters": {"preconditioner": "multigrid", "stagnation_tolerance": 1e-3,
                                 "max_shift_attempts": 5, "shift_multiplier": 4.0, "mg_levels": 4,
                                 "smoother_sweeps": 3, "use_cuda_graphs": False}, "force_float64": True}
    p = params_from_config(cfg, nu=0.3, tol=1e-9, max_iter=30000, shift_factor=1e-10)
    assert p.precond == 1 and p.stagnation_tol == 1e-3 and p.max_shift_attempts == 5 and p.shift_multiplier == 4.0
    assert p.mg_levels == 4 and p.pre_smooth == 3 and p.post_smooth == 3 and p.use_graphs == 0 and p.precision == 0


def test_workload_generators():
    f = workloads.edge_load(48, 24, 24)
    assert f.sum() == pytest.approx(-1.0) and np.count_nonzero(f) == 25
    rho = workloads.c1_density()
    assert rho.size == 27648 and rho.min() >= 0.25 and rho.max() <= 0.35
    assert np.array_equal(rho, workloads.c1_density())
    r2 = workloads.smooth_density(16, 8, 8, lambda g, R: g)
    assert abs(r2.mean() - 0.3) < 1e-12 and r2.min() >= 0.001 and r2.max() <= 1.0
    F = workloads.point_loads(16, 8, 8, 8)
    assert F.shape == (8, 3 * 17 * 9 * 9) and np.allclose(np.linalg.norm(F, axis=1), 1.0)
    sizes = workloads.batch_sizes()
    assert len(sizes) == 64 and all(16 <= s[0] <= 96 and s[0] % 8 == 0 and s[1] == s[0] // 2 for s in sizes)
