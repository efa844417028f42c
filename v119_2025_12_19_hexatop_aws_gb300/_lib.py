"""ctypes binding of libhexagpu.so (the C ABI declared in include/hexagpu.h).

The library is built in-tree by ``build.py``.  Loading fails loudly when the
shared object is missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libhexagpu.so"

HEXA_OK = 0
HEXA_NOT_CONVERGED = 1
HEXA_ERR_ARG = -1
HEXA_ERR_CUDA = -2
HEXA_ERR_NOMEM = -3
HEXA_ERR_CORRUPT_INPUT = -4
HEXA_ERR_NO_DEVICE = -5
HEXA_ERR_TOO_LARGE = -6
NOALLOC_MAX_NODES = 262144

PRECOND = {"jacobi": 0, "multigrid": 1}
PRECISION = {"fp64": 0, "mixed": 1, "fp32": 2}
SMOOTHER = {"jacobi": 0, "chebyshev": 1}


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class BC(C.Structure):
    _fields_ = [("clamp_faces", C.c_uint32), ("fixed_dof", C.c_void_p)]


class SolveParams(C.Structure):
    _fields_ = [
        ("nu", C.c_double), ("tol", C.c_double), ("max_iter", C.c_int32), ("precond", C.c_int32),
        ("shift_factor", C.c_double), ("stagnation_tol", C.c_double), ("max_shift_attempts", C.c_int32),
        ("shift_multiplier", C.c_double), ("check_cadence", C.c_int32), ("diag_quirk", C.c_int32),
        ("precision", C.c_int32), ("mg_levels", C.c_int32), ("pre_smooth", C.c_int32), ("post_smooth", C.c_int32),
        ("smoother", C.c_int32), ("jacobi_omega", C.c_double), ("cheb_ratio", C.c_int32),
        ("coarse_iters", C.c_int32), ("inner_tol", C.c_double), ("max_outer", C.c_int32),
        ("use_graphs", C.c_int32), ("graph_iters", C.c_int32), ("true_residual", C.c_int32),
        ("divergence_check", C.c_int32), ("autotune", C.c_int32), ("mg_cycle", C.c_int32),
    ]


class SolveStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("iterations", C.c_int32), ("outer_iterations", C.c_int32), ("attempts", C.c_int32),
        ("precond_used", C.c_int32), ("mg_levels", C.c_int32), ("smooth_steps", C.c_int32), ("relres", C.c_double),
        ("true_relres", C.c_double),
        ("shift", C.c_double), ("max_diag", C.c_double), ("compliance", C.c_double), ("setup_ms", C.c_double),
        ("solve_ms", C.c_double), ("total_ms", C.c_double), ("fine_applies", C.c_double),
        ("fine_applies_fp64", C.c_double), ("unshifted_relres", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class FilterStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32), ("relres", C.c_double), ("solve_ms", C.c_double)]


class DensityUpdateParams(C.Structure):
    _fields_ = [("E", C.c_float), ("l1_stress_allowable", C.c_float), ("iter", C.c_int32),
                ("number_of_iterations", C.c_int32), ("min_density", C.c_float), ("max_density", C.c_float),
                ("max_domain_dim", C.c_float), ("filter_R_init_perc", C.c_float), ("filter_R_interm_perc", C.c_float),
                ("filter_R_final_perc", C.c_float), ("filter_R_interm_iter_perc", C.c_float),
                ("minimum_filter_radius_as_elements", C.c_float), ("filter_tolerance", C.c_float),
                ("final_density_threshold", C.c_float), ("max_culling_ratio", C.c_float), ("hard_update", C.c_int32),
                ("filter_max_iter", C.c_int32), ("filter_precision", C.c_int32)]


class DensityUpdateStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("filter_used", C.c_int32), ("filter_nan_fallback", C.c_int32),
                ("filter_iters", C.c_int32), ("mean_change", C.c_float), ("R_length", C.c_float),
                ("current_threshold", C.c_float), ("R_effective", C.c_float), ("filter_time", C.c_double),
                ("filter_res", C.c_double), ("active_count", C.c_int64), ("candidates", C.c_int64),
                ("culled", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
D = C.c_double
I32 = C.c_int32
I64 = C.c_int64

# name -> (restype, argtypes); every symbol include/hexagpu.h declares
SIGNATURES = {
    "hexa_create": (I32, [I32, C.POINTER(P)]),
    "hexa_destroy": (None, [P]),
    "hexa_last_error": (C.c_char_p, [P]),
    "hexa_version": (I32, []),
    "hexa_default_params": (None, [C.POINTER(SolveParams)]),
    "hexa_last_device_ms": (D, [P]),
    "hexa_kernel_launches": (I64, [P]),
    "hexa_canonical_stiffness": (I32, [D, D, D, D, P]),
    "hexa_scalar_canonical_matrices": (I32, [D, D, D, I32, P, P]),
    "hexa_apply_operator": (I32, [P, C.POINTER(Grid), C.POINTER(BC), D, P, P, D, P]),
    "hexa_apply_operator_f32": (I32, [P, C.POINTER(Grid), C.POINTER(BC), D, P, P, C.c_float, P]),
    "hexa_time_operator": (I32, [P, C.POINTER(Grid), C.POINTER(BC), D, I32, I32, P, P, P, P, I32, C.POINTER(D)]),
    "hexa_operator_diagonal": (I32, [P, C.POINTER(Grid), C.POINTER(BC), D, P, I32, P]),
    "hexa_solve": (I32, [P, C.POINTER(Grid), C.POINTER(BC), P, P, C.POINTER(SolveParams), P, P,
                         C.POINTER(SolveStats)]),
    "hexa_solve_system_gpu": (I32, [P, C.POINTER(Grid), C.c_float, P, P, P, C.POINTER(SolveParams), P, P,
                                    C.POINTER(D), C.c_char_p, I32, C.POINTER(SolveStats)]),
    "hexa_solve_system": (I32, [P, C.POINTER(Grid), C.c_float, P, P, P, C.c_float, I32, I32, C.POINTER(SolveParams),
                                P, P, C.POINTER(D), C.c_char_p, I32, C.POINTER(SolveStats), C.POINTER(I64)]),
    "hexa_solve_multi_rhs": (I32, [P, C.POINTER(Grid), C.POINTER(BC), P, I32, P, C.POINTER(SolveParams), P,
                                   C.POINTER(SolveStats)]),
    "hexa_solve_batch": (I32, [P, I32, C.POINTER(Grid), C.POINTER(BC), D, C.POINTER(P), C.POINTER(P),
                               C.POINTER(SolveParams), C.POINTER(P), C.POINTER(SolveStats)]),
    "hexa_filter": (I32, [P, C.POINTER(Grid), P, D, D, I32, I32, I32, P, C.POINTER(FilterStats)]),
    "hexa_filter_batch": (I32, [P, I32, C.POINTER(Grid), C.POINTER(P), D, D, I32, I32, I32, C.POINTER(P),
                                C.POINTER(FilterStats)]),
    "hexa_filter_noalloc": (I32, [C.POINTER(Grid), P, D, D, I32, I32, P, P, C.POINTER(FilterStats)]),
    "hexa_remap_displacement": (I32, [P, C.POINTER(Grid), C.POINTER(Grid), P, P]),
    "hexa_remap_fields": (I32, [P, C.POINTER(Grid), C.POINTER(Grid), D, D, D, P, P, I32, P, P]),
    "hexa_default_density_update_params": (None, [C.POINTER(DensityUpdateParams)]),
    "hexa_update_density": (I32, [P, C.POINTER(Grid), P, P, P, P, C.POINTER(DensityUpdateParams),
                                  C.POINTER(DensityUpdateStats)]),
    "hexa_stress_field": (I32, [P, C.POINTER(Grid), P, P, C.c_float, C.c_float, P, P, P, P, P, P]),
    "hexa_sensitivities": (I32, [P, C.POINTER(Grid), D, P, P, D, D, D, P, C.POINTER(D)]),
    "hexa_simp_factors": (I32, [P, I64, P, D, D, D, P]),
    "hexa_oc_update": (I32, [P, I64, P, P, P, D, D, P, C.POINTER(D)]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libhexagpu.so and bind every exported symbol; raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -m v119_2025_12_19_hexatop_aws_gb300.build` "
            "(this package has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def ptr(a) -> int | None:
    """Address of a numpy array (host) or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays passed to libhexagpu must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError("tensors passed to libhexagpu must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)!r}")


class HexaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libhexagpu error {code}: {msg}")
        self.code = code


class Context:
    """One library context (stream, cached workspaces) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = P()
        rc = self.lib.hexa_create(int(device), C.byref(h))
        if rc != HEXA_OK:
            raise HexaError(rc, "hexa_create failed (no usable CUDA device?)")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.hexa_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def error(self) -> str:
        s = self.lib.hexa_last_error(self.h)
        return s.decode() if s else ""

    def check(self, rc: int, allow=(HEXA_OK, HEXA_NOT_CONVERGED)) -> int:
        if rc not in allow:
            raise HexaError(rc, self.error())
        return rc

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.hexa_kernel_launches(self.h))

    @property
    def last_device_ms(self) -> float:
        return float(self.lib.hexa_last_device_ms(self.h))


def default_params(**kw) -> SolveParams:
    p = SolveParams()
    load().hexa_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "precond" and isinstance(v, str):
            v = PRECOND[v]
        if k == "precision" and isinstance(v, str):
            v = PRECISION[v]
        if k == "smoother" and isinstance(v, str):
            v = SMOOTHER[v]
        if not hasattr(p, k):
            raise KeyError(f"unknown solver parameter {k!r}")
        setattr(p, k, v)
    return p


def make_grid(nx, ny, nz, dx=1.0, dy=1.0, dz=1.0) -> Grid:
    return Grid(int(nx), int(ny), int(nz), float(dx), float(dy), float(dz))


def make_bc(clamp_faces: int = 0, fixed_dof: np.ndarray | None = None) -> BC:
    b = BC()
    b.clamp_faces = int(clamp_faces)
    b.fixed_dof = ptr(fixed_dof) if fixed_dof is not None else None
    b._keep = fixed_dof  # keep the buffer alive with the struct
    return b


def exported_symbols() -> list[str]:
    return list(SIGNATURES)


if os.environ.get("HEXA_EAGER_LOAD"):
    load()
