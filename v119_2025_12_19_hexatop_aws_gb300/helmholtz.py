"""Host-side mirror of ``GPUHelmholtz.apply_gpu_filter!``.

Same arguments, same ``(filtered, time, iters, res)`` return and the same
failure convention (an empty vector, src/Optimization/GPUHelmholtz.jl:436-442)
for solver errors; a missing libhexagpu.so raises instead of falling back to a
CPU filter.  ``radius`` is the Helmholtz length R of (R^2 K_s + M_s) psi = b;
the reference's caller maps its filter length with R = R_length / 2.5
(src/Optimization/TopOpt.jl:300), see ``radius_from_length``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .solver import context


def radius_from_length(R_length: float) -> float:
    """R_effective = R_length / 2.5 (TopOpt.jl:300)."""
    return float(np.float32(R_length) / np.float32(2.5))


def filter_density(grid: _lib.Grid, rho, radius: float, *, tol: float = 1e-5, max_iter: int = 200, quirk: bool = True,
                   precision: str = "fp64", out=None, ctx=None):
    """rho_tilde = element mean of psi, (R^2 K_s + M_s) psi = sum_e rho_e vol/8.

    Returns (out, stats dict).  quirk=True keeps the reference's element
    geometry (top face at +dz, Element.jl:116); quirk=False uses the true
    brick, for which a constant field is preserved exactly."""
    ctx = ctx or context()
    ne = grid.nx * grid.ny * grid.nz
    if out is None:
        out = np.empty(ne, dtype=np.float64)
    st = _lib.FilterStats()
    rc = ctx.lib.hexa_filter(ctx.h, C.byref(grid), _lib.ptr(rho), float(radius), float(tol), int(max_iter),
                             int(bool(quirk)), _lib.PRECISION[precision], _lib.ptr(out), C.byref(st))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return out, {"iterations": st.iterations, "relres": st.relres, "solve_ms": st.solve_ms}


def filter_batch(grids, rhos, radius: float, *, tol: float = 1e-5, max_iter: int = 200, quirk: bool = True,
                 precision: str = "fp64", out=None, ctx: _lib.Context | None = None):
    """The filter of filter_density over grids of uneven sizes in one batch.
    Returns (list of filtered densities, list of stats dicts)."""
    ctx = ctx or context()
    n = len(grids)
    if len(rhos) != n or n < 1:
        raise ValueError("grids and rhos must have the same (non-zero) length")
    if out is None:
        out = [np.empty(g.nx * g.ny * g.nz) for g in grids]
    G = (_lib.Grid * n)(*grids)
    rp = (C.c_void_p * n)(*[_lib.ptr(a) for a in rhos])
    op = (C.c_void_p * n)(*[_lib.ptr(a) for a in out])
    st = (_lib.FilterStats * n)()
    rc = ctx.lib.hexa_filter_batch(ctx.h, n, G, rp, float(radius), float(tol), int(max_iter), int(bool(quirk)),
                                   _lib.PRECISION[precision], op, st)
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return out, [{"iterations": st[i].iterations, "relres": st[i].relres, "solve_ms": st[i].solve_ms}
                 for i in range(n)]


def apply_gpu_filter(density_cpu, nElem_x, nElem_y, nElem_z, dx, dy, dz, radius, elements_cpu=None, tol=1.0e-5,
                     *, quirk=True, precision="fp32", max_iter=200):
    """Drop-in for apply_gpu_filter! (GPUHelmholtz.jl:422-443).

    The reference solves in Float32 (its workspace type); precision="fp64"
    gives the FP64 form.  Returns (filtered::Float32 or Float64, time_s, iters, res)."""
    grid = _lib.make_grid(nElem_x, nElem_y, nElem_z, dx, dy, dz)
    rho = np.ascontiguousarray(np.asarray(density_cpu, dtype=np.float64))
    try:
        out, st = filter_density(grid, rho, float(radius), tol=float(tol), max_iter=max_iter, quirk=quirk,
                                 precision=precision)
    except _lib.HexaError as e:  # reference: print and return an empty vector
        print(f"  [GPU Filter] CRITICAL ERROR: {e}.")
        return np.zeros(0, dtype=np.float32), 0.0, 0, 0.0
    dt = np.float32 if precision == "fp32" else np.float64
    return out.astype(dt), st["solve_ms"] / 1e3, st["iterations"], st["relres"]
