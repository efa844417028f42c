"""GB300-native finite-element solve path of HEXA TopOpt.

A C-ABI shared library (libhexagpu.so, include/hexagpu.h) with hand-written
sm_103a kernels for the matrix-free hex8 operator, fused PCG passes, a
geometric-multigrid V-cycle, the Helmholtz density filter and SIMP
sensitivities / OC updates; this package is the host-side mirror of the
reference's entry points (GPUSolver.solve_system_gpu, Solver.solve_system,
GPUHelmholtz.apply_gpu_filter!) on top of it.
"""
from . import _lib
from ._lib import Context, HexaError, default_params, make_grid
from .helmholtz import apply_gpu_filter, filter_density, radius_from_length
from .mesh import generate_mesh, node_index, structured_dims
from .solver import apply_operator, canonical_stiffness, operator_diagonal, solve, solve_system, solve_system_gpu

__all__ = [
    "Context", "HexaError", "default_params", "make_grid", "apply_gpu_filter", "filter_density",
    "radius_from_length", "generate_mesh", "node_index", "structured_dims", "apply_operator",
    "canonical_stiffness", "operator_diagonal", "solve", "solve_system", "solve_system_gpu",
]
