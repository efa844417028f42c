"""SIMP compliance minimisation with OC updates on the GPU path.

The reference's optimiser is a stress-ratio / cull rule with a modulus linear
in density (src/Optimization/TopOpt.jl:211-482, src/Solvers/GPUSolver.jl:254).
The benchmark loop instead is the published SIMP + OC method (Andreassen et
al. 2011, with the Helmholtz PDE filter of Lazarov & Sigmund 2011) and
reaches the same solve call with the SIMP modulus as the element factor:

    xPhys = F(x)                      (Helmholtz filter, true brick geometry)
    E_e   = Emin + xPhys_e^p (E0 - Emin)
    u     = solve (K(E) + sigma I) u = f
    c     = sum_e E_e u_e^T K0 u_e,  dc_e = -p xPhys^(p-1) (E0-Emin) u_e^T K0 u_e
    dc_x  = F(dc), dv_x = F(1)        (F is symmetric, so this is the chain rule)
    x     = OC(x, dc_x, dv_x)         (bisection on lambda, move limit)

With the true brick F preserves the mean, so the volume test on x equals the
test on xPhys.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .helmholtz import filter_density
from .solver import context, solve


def simp_factors(rho, Emin=1e-9, E0=1.0, penal=3.0, ctx=None):
    ctx = ctx or context()
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    out = np.empty_like(rho)
    ctx.check(ctx.lib.hexa_simp_factors(ctx.h, rho.size, _lib.ptr(rho), Emin, E0, penal, _lib.ptr(out)),
              allow=(_lib.HEXA_OK,))
    return out


def sensitivities(grid, rho, u, *, nu=0.3, Emin=1e-9, E0=1.0, penal=3.0, ctx=None):
    """(dc, compliance) for element densities rho and displacements u."""
    ctx = ctx or context()
    dc = np.empty(grid.nx * grid.ny * grid.nz, dtype=np.float64)
    c = C.c_double(0.0)
    rc = ctx.lib.hexa_sensitivities(ctx.h, C.byref(grid), float(nu), _lib.ptr(rho), _lib.ptr(u), Emin, E0, penal,
                                    _lib.ptr(dc), C.byref(c))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return dc, c.value


def oc_update(x, dc, dv, volfrac, move=0.2, ctx=None):
    ctx = ctx or context()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lam = C.c_double(0.0)
    rc = ctx.lib.hexa_oc_update(ctx.h, x.size, _lib.ptr(x), _lib.ptr(np.ascontiguousarray(dc)),
                                _lib.ptr(np.ascontiguousarray(dv)), float(volfrac), float(move), _lib.ptr(out),
                                C.byref(lam))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return out, lam.value


@dataclass
class SimpSetup:
    grid: _lib.Grid
    f: np.ndarray
    clamp_faces: int = 1
    fixed_dof: np.ndarray | None = None
    nu: float = 0.3
    Emin: float = 1e-9
    E0: float = 1.0
    penal: float = 3.0
    volfrac: float = 0.3
    filter_radius: float = 0.6      # Helmholtz R (elements * dx / 2.5 by the reference convention)
    filter_tol: float = 1e-12
    move: float = 0.2
    params: _lib.SolveParams | None = None


@dataclass
class SimpRecord:
    compliance: float
    volume: float
    iterations: int
    true_relres: float
    u: np.ndarray = field(repr=False)
    dc: np.ndarray = field(repr=False)
    xphys: np.ndarray = field(repr=False)
    unshifted_relres: float = float("nan")  # ||f - K u|| / ||f|| in FP64, without the diagonal shift


def run_simp(S: SimpSetup, x0: np.ndarray, n_iter: int = 10, keep=True, ctx=None) -> list[SimpRecord]:
    ctx = ctx or context()
    x = np.ascontiguousarray(x0, dtype=np.float64)
    ne = x.size
    ones = np.ones(ne)
    dv, _ = filter_density(S.grid, ones, S.filter_radius, tol=S.filter_tol, quirk=False, max_iter=10000, ctx=ctx)
    hist = []
    u = None
    for _ in range(n_iter):
        xphys, _ = filter_density(S.grid, x, S.filter_radius, tol=S.filter_tol, quirk=False, max_iter=10000, ctx=ctx)
        fac = simp_factors(xphys, S.Emin, S.E0, S.penal, ctx=ctx)
        params = S.params or _lib.default_params(divergence_check=0)
        u, st = solve(S.grid, fac, S.f, clamp_faces=S.clamp_faces, fixed_dof=S.fixed_dof, params=params, ctx=ctx)
        dc, c = sensitivities(S.grid, xphys, u, nu=S.nu, Emin=S.Emin, E0=S.E0, penal=S.penal, ctx=ctx)
        dcx, _ = filter_density(S.grid, dc, S.filter_radius, tol=S.filter_tol, quirk=False, max_iter=10000, ctx=ctx)
        hist.append(SimpRecord(c, float(xphys.mean()), int(st["iterations"]), float(st["true_relres"]),
                               u.copy() if keep else None, dc.copy() if keep else None,
                               xphys.copy() if keep else None, float(st["unshifted_relres"])))
        x, _ = oc_update(x, dcx, dv, S.volfrac, S.move, ctx=ctx)
    return hist


def stress_field(grid, u, density, *, E=1.0, nu=0.3, voigt=True, ctx=None):
    """Stress.compute_stress_field (Stress.jl:286-339) on the GPU: per element
    principal stresses (descending), von Mises, Voigt stress, L1 norm of the
    principal stresses and the directions of the largest and smallest.
    Returns a dict of float32 arrays, element-major (principal[e, i])."""
    ctx = ctx or context()
    ne = grid.nx * grid.ny * grid.nz
    out = dict(principal=np.empty((ne, 3), np.float32), vonmises=np.empty(ne, np.float32),
               voigt=np.empty((ne, 6), np.float32) if voigt else None, l1=np.empty(ne, np.float32),
               dir_max=np.empty((ne, 3), np.float32), dir_min=np.empty((ne, 3), np.float32))
    rc = ctx.lib.hexa_stress_field(ctx.h, C.byref(grid), _lib.ptr(np.ascontiguousarray(u, dtype=np.float64)),
                                   _lib.ptr(np.ascontiguousarray(density, dtype=np.float32)), float(E), float(nu),
                                   _lib.ptr(out["principal"]), _lib.ptr(out["vonmises"]), _lib.ptr(out["voigt"]),
                                   _lib.ptr(out["l1"]), _lib.ptr(out["dir_max"]), _lib.ptr(out["dir_min"]))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return out


def density_update_params(**kw) -> _lib.DensityUpdateParams:
    """hexa_density_update_params with the library defaults, fields overridden by keyword."""
    p = _lib.DensityUpdateParams()
    _lib.load().hexa_default_density_update_params(C.byref(p))
    names = {f for f, _ in p._fields_}
    for k, v in kw.items():
        if k not in names:
            raise KeyError(k)
        setattr(p, k, v)
    return p


def update_density_gpu(grid, density, l1, protected, original, params, *, ctx=None):
    """hexa_update_density: density (float32 numpy array or device tensor) is
    updated in place; returns the statistics as a dict."""
    ctx = ctx or context()
    if isinstance(density, np.ndarray) and (density.dtype != np.float32 or not density.flags.c_contiguous):
        raise TypeError("density must be a contiguous float32 array (it is updated in place)")
    def f32(a):  # numpy arrays are converted; tensors (host or device) are passed as they are
        return a if hasattr(a, "data_ptr") else np.ascontiguousarray(a, dtype=np.float32)

    prot = None if protected is None else np.ascontiguousarray(np.asarray(protected, dtype=bool).view(np.uint8))
    st = _lib.DensityUpdateStats()
    l1a, oa = f32(l1), f32(original)
    rc = ctx.lib.hexa_update_density(ctx.h, C.byref(grid), _lib.ptr(density), _lib.ptr(l1a), _lib.ptr(prot),
                                     _lib.ptr(oa), C.byref(params), C.byref(st))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return st.as_dict()


def update_density(density, l1_stress_norm_field, protected_elements_mask, E, l1_stress_allowable, iter,
                   number_of_iterations, original_density, min_density, max_density, config, elements=None,
                   is_annealing=False, *, ctx=None):
    """Drop-in for TopologyOptimization.update_density! (TopOpt.jl:211-482):
    same arguments and config keys, density (float32) updated in place,
    returns (mean_change, R_length, current_threshold, filter_time,
    filter_iters, filter_res).  The structured grid comes from the config's
    geometry.{nElem,d}{x,y,z}_computed; `elements` is not needed."""
    opt = config["optimization_parameters"]
    geom = config["geometry"]
    solver = config.get("solver_parameters", {})
    grid = _lib.make_grid(int(geom["nElem_x_computed"]), int(geom["nElem_y_computed"]), int(geom["nElem_z_computed"]),
                          float(np.float32(geom["dx_computed"])), float(np.float32(geom["dy_computed"])),
                          float(np.float32(geom["dz_computed"])))
    p = density_update_params(
        E=float(E), l1_stress_allowable=float(l1_stress_allowable), iter=int(iter),
        number_of_iterations=int(number_of_iterations), min_density=float(min_density),
        max_density=float(max_density), max_domain_dim=float(geom["max_domain_dim"]),
        filter_R_init_perc=float(opt.get("filter_R_init_perc", 0.0)),
        filter_R_interm_perc=float(opt.get("filter_R_interm_perc", 0.0)),
        filter_R_final_perc=float(opt.get("filter_R_final_perc", 0.0)),
        filter_R_interm_iter_perc=float(opt.get("filter_R_interm_iter_perc", 50.0)),
        minimum_filter_radius_as_elements=float(opt.get("minimum_filter_radius_as_elements", 2.5)),
        filter_tolerance=float(solver.get("filter_tolerance", 1.0e-5)),
        final_density_threshold=float(opt.get("final_density_threshold", 0.95)),
        max_culling_ratio=float(opt.get("max_culling_ratio", 0.1)),
        hard_update=int(opt.get("density_update_method", "soft") == "hard"))
    st = update_density_gpu(grid, density, l1_stress_norm_field, protected_elements_mask, original_density, p, ctx=ctx)
    if st["status"] == 1:
        return np.float32(0), np.float32(0), np.float32(0), 0.0, 0, 0.0
    return (np.float32(st["mean_change"]), np.float32(st["R_length"]), np.float32(st["current_threshold"]),
            st["filter_time"], st["filter_iters"], st["filter_res"])


def compute_stress_field(nodes, elements, U, E, nu, density, *, return_voigt=True, ctx=None):
    """Drop-in for Stress.compute_stress_field (Stress.jl:286-339) on a mesh
    that equals Mesh.generate_mesh's: returns (principal, vonmises, voigt,
    l1, dir_max, dir_min) as the reference does, the 3 x nElem and 6 x nElem
    matrices as (3, nElem) / (6, nElem) views of the element-major arrays
    (the memory layout of the reference's column-major matrices); voigt is an
    empty (0, 0) array when return_voigt is false."""
    from .mesh import structured_dims
    nx, ny, nz, dx, dy, dz = structured_dims(nodes, elements)
    grid = _lib.make_grid(nx, ny, nz, dx, dy, dz)
    out = stress_field(grid, np.asarray(U, dtype=np.float64), density, E=float(E), nu=float(nu), voigt=return_voigt,
                       ctx=ctx)
    voigt = out["voigt"].T if return_voigt else np.zeros((0, 0), np.float32)
    return out["principal"].T, out["vonmises"], voigt, out["l1"], out["dir_max"].T, out["dir_min"].T
