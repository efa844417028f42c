"""Host-side mirror of the reference's solve entry points.

``solve_system_gpu`` keeps the signature, argument meaning and return
convention of ``GPUSolver.solve_system_gpu`` (src/Solvers/GPUSolver.jl:467-477)
and ``solve_system`` those of ``Solver.solve_system`` for the ``gpu`` solver
type (src/Solvers/Solver.jl:39-160).  Both reach the C ABI (libhexagpu.so);
there is no CPU path behind them.

Config keys read (configs/default.yaml:209-237, GPUSolver.jl:187-231):
``solver_parameters.{tolerance, max_iterations, diagonal_shift_factor,
preconditioner, stagnation_tolerance, max_shift_attempts, shift_multiplier}``,
``hardware_profile_applied`` / ``force_float64`` (precision) and
``geometry.d*_computed``.  Optional new keys under ``solver_parameters``:
``precision`` (fp64 | mixed | fp32), ``mg_levels``, ``smoother_sweeps``,
``jacobi_omega``, ``coarse_iterations``, ``inner_tolerance``,
``use_cuda_graphs``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .boundary import bc_to_fixed_dof, face_clamps
from .mesh import structured_dims

_CTX: _lib.Context | None = None


def context(device: int = 0) -> _lib.Context:
    """Process-wide context, like the reference's GLOBAL_CG_CACHE (GPUSolver.jl:63)."""
    global _CTX
    if _CTX is None or _CTX.h is None:
        _CTX = _lib.Context(device)
    return _CTX


def precision_from_config(config: dict) -> str:
    """GPUSolver.jl:187-189: FP64 for the H200/V100/A100 profiles or force_float64."""
    sp = config.get("solver_parameters", {}) or {}
    if "precision" in sp:
        return str(sp["precision"]).lower()
    prof = config.get("hardware_profile_applied", "RTX")
    use_double = prof in ("H200", "V100", "A100") or bool(config.get("force_float64", False))
    return "fp64" if use_double else "fp32"


def params_from_config(config: dict, *, nu: float, tol: float, max_iter: int, shift_factor: float) -> _lib.SolveParams:
    sp = config.get("solver_parameters", {}) or {}
    kw = dict(
        nu=float(nu), tol=float(tol), max_iter=int(max_iter), shift_factor=float(shift_factor),
        precond="multigrid" if str(sp.get("preconditioner", "jacobi")).lower() == "multigrid" else "jacobi",
        stagnation_tol=float(sp.get("stagnation_tolerance", 0.0)),
        max_shift_attempts=int(sp.get("max_shift_attempts", 3)),
        shift_multiplier=float(sp.get("shift_multiplier", 10.0)),
        precision=precision_from_config(config),
    )
    opt = {"mg_levels": "mg_levels", "jacobi_omega": "jacobi_omega", "coarse_iterations": "coarse_iters",
           "inner_tolerance": "inner_tol", "check_cadence": "check_cadence", "diag_quirk": "diag_quirk",
           "graph_iterations": "graph_iters"}
    for key, field in opt.items():
        if key in sp:
            kw[field] = sp[key]
    if "smoother_sweeps" in sp:
        kw["pre_smooth"] = kw["post_smooth"] = int(sp["smoother_sweeps"])
    if "use_cuda_graphs" in sp:
        kw["use_graphs"] = int(bool(sp["use_cuda_graphs"]))
    return _lib.default_params(**kw)


def solve(grid: _lib.Grid, factor, f, *, clamp_faces: int = 0, fixed_dof=None, params: _lib.SolveParams | None = None,
          u_guess=None, u_out=None, ctx: _lib.Context | None = None):
    """Solve (K_ff(factor) + sigma I) u = f_free on the structured grid.

    factor: nElem modulus factors (float64); f: 3*nNodes forces (float64);
    arrays may be numpy (host) or torch CUDA tensors (device, used in place).
    Returns (u, stats dict)."""
    ctx = ctx or context()
    params = params or _lib.default_params()
    ndof = 3 * (grid.nx + 1) * (grid.ny + 1) * (grid.nz + 1)
    if u_out is None:
        u_out = np.empty(ndof, dtype=np.float64)
    bc = _lib.make_bc(clamp_faces, fixed_dof)
    st = _lib.SolveStats()
    rc = ctx.lib.hexa_solve(ctx.h, C.byref(grid), C.byref(bc), _lib.ptr(factor), _lib.ptr(f), C.byref(params),
                            _lib.ptr(u_guess), _lib.ptr(u_out), C.byref(st))
    ctx.check(rc)
    return u_out, st.as_dict()


def solve_multi_rhs(grid: _lib.Grid, factor, F, *, clamp_faces: int = 0, fixed_dof=None,
                    params: _lib.SolveParams | None = None, U_out=None, ctx: _lib.Context | None = None):
    """Solve the k load cases F (k x 3*nNodes, row j = load case j) as one block PCG.

    precision "fp64": block PCG in FP64; "mixed"/"fp32": FP32 block PCG with
    FP64 reliable updates to params.tol per column.  Returns (U, stats dict);
    stats["compliance"] is the sum over the load cases of f_j . u_j and
    stats["true_relres"] the largest per-column FP64 relative residual."""
    ctx = ctx or context()
    params = params or _lib.default_params()
    ndof = 3 * (grid.nx + 1) * (grid.ny + 1) * (grid.nz + 1)
    k = int(F.shape[0])
    if tuple(F.shape) != (k, ndof):
        raise ValueError(f"F must have shape (k, {ndof})")
    if U_out is None:
        U_out = np.empty((k, ndof), dtype=np.float64)
    bc = _lib.make_bc(clamp_faces, fixed_dof)
    st = _lib.SolveStats()
    rc = ctx.lib.hexa_solve_multi_rhs(ctx.h, C.byref(grid), C.byref(bc), _lib.ptr(factor), k, _lib.ptr(F),
                                      C.byref(params), _lib.ptr(U_out), C.byref(st))
    ctx.check(rc)
    return U_out, st.as_dict()


def solve_batch(grids, factors, forces, *, clamp_faces=0, nu: float = 0.3, params: _lib.SolveParams | None = None,
                u_out=None, ctx: _lib.Context | None = None):
    """Solve independent problems on grids of uneven sizes in one batch.

    grids: list of _lib.Grid (same element size); factors[i] (nElem_i) and
    forces[i] (3*nNodes_i) float64 numpy arrays or CUDA tensors; clamp_faces an
    int for all instances or one per instance.  Mixed precision GMG-PCG.
    Returns (list of u, list of stats dicts, status)."""
    ctx = ctx or context()
    params = params or _lib.default_params(precision="mixed", precond="multigrid")
    n = len(grids)
    if not (len(factors) == len(forces) == n) or n < 1:
        raise ValueError("grids, factors and forces must have the same (non-zero) length")
    faces = [clamp_faces] * n if np.isscalar(clamp_faces) else list(clamp_faces)
    if u_out is None:
        u_out = [np.empty(3 * (g.nx + 1) * (g.ny + 1) * (g.nz + 1)) for g in grids]
    G = (_lib.Grid * n)(*grids)
    bcs = (_lib.BC * n)(*[_lib.make_bc(fc) for fc in faces])
    fac_p = (C.c_void_p * n)(*[_lib.ptr(a) for a in factors])
    f_p = (C.c_void_p * n)(*[_lib.ptr(a) for a in forces])
    u_p = (C.c_void_p * n)(*[_lib.ptr(a) for a in u_out])
    st = (_lib.SolveStats * n)()
    rc = ctx.lib.hexa_solve_batch(ctx.h, n, G, bcs, float(nu), fac_p, f_p, C.byref(params), u_p, st)
    ctx.check(rc)
    return u_out, [st[i].as_dict() for i in range(n)], rc


def solve_system_gpu(nodes, elements, E, nu, bc, f, density, *, max_iter=40000, tol=1e-6, method="native",
                     solver="cg", use_precond=True, shift_factor=1.0e-4, min_stiffness_threshold=1.0e-3,
                     u_guess=None, config=None):
    """Drop-in for GPUSolver.solve_system_gpu: returns (u::Float64[3nNodes], relres, name).

    name is "GMG_GPU", "Jacobi_GPU" or "Failed_Corrupt_Input" (GPUSolver.jl:314,463)."""
    config = config or {}
    nx, ny, nz, dx, dy, dz = structured_dims(nodes, elements)
    geom = config.get("geometry", {}) or {}
    dx = float(geom.get("dx_computed", dx))
    dy = float(geom.get("dy_computed", dy))
    dz = float(geom.get("dz_computed", dz))
    grid = _lib.make_grid(nx, ny, nz, dx, dy, dz)
    params = params_from_config(config, nu=nu, tol=tol, max_iter=max_iter, shift_factor=shift_factor)
    ctx = context()
    fixed = bc_to_fixed_dof(bc)
    faces, rest = face_clamps(fixed, nx, ny, nz)
    # the reference promotes Float32(E*density) (GPUSolver.jl:254)
    factor = (np.float32(E) * np.asarray(density, dtype=np.float32)).astype(np.float64)
    fvec = np.ascontiguousarray(np.asarray(f, dtype=np.float32).astype(np.float64))
    guess = None
    if u_guess is not None and len(u_guess) > 0:
        guess = np.ascontiguousarray(np.asarray(u_guess, dtype=np.float64))
    u = np.empty(3 * (nx + 1) * (ny + 1) * (nz + 1), dtype=np.float64)
    bcs = _lib.make_bc(faces, rest)
    st = _lib.SolveStats()
    rc = ctx.lib.hexa_solve(ctx.h, C.byref(grid), C.byref(bcs), _lib.ptr(factor), _lib.ptr(fvec), C.byref(params),
                            _lib.ptr(guess), _lib.ptr(u), C.byref(st))
    if rc == _lib.HEXA_ERR_CORRUPT_INPUT:
        return np.zeros(u.shape[0], dtype=np.float64), float("nan"), "Failed_Corrupt_Input"
    ctx.check(rc)
    name = "GMG_GPU" if st.precond_used == 1 else "Jacobi_GPU"
    return u, float(st.relres), name


def solve_system(nodes, elements, E, nu, bc_indicator, F, *, density, config, min_stiffness_threshold=1.0e-3,
                 prune_voids=True, u_prev=None, stats=None):
    """Solver.solve_system for solver_type "gpu" (Solver.jl:39-160): returns
    (U_full, relres, name).

    The tolerance and shift factor are cast to Float32 as the reference does
    (Solver.jl:57-59).  Void pruning keeps the reference's rule (from
    config["current_outer_iter"] 3 on, when fewer than 99 % of the elements
    have density > 1.01 min_stiffness_threshold, MeshPruner.jl:10-87): the
    library solves the pruned system on the structured grid (removed elements'
    factors zero, removed nodes' DOFs fixed) and U_full is zero at removed
    nodes, as reconstruct_full_solution writes.  `stats`, when a dict, receives
    the solve statistics and the number of elements in the solved system."""
    sp = config["solver_parameters"]
    stype = str(sp.get("solver_type", "direct")).lower()
    if stype != "gpu":
        raise NotImplementedError(f"solver_type {stype!r}: this library implements the 'gpu' solve path only")
    tol = float(np.float32(sp.get("tolerance", 1.0e-6)))
    max_iter = int(sp.get("max_iterations", 1000))
    shift = float(np.float32(sp.get("diagonal_shift_factor", 1.0e-6)))
    nx, ny, nz, dx, dy, dz = structured_dims(nodes, elements)
    geom = config.get("geometry", {}) or {}
    grid = _lib.make_grid(nx, ny, nz, float(geom.get("dx_computed", dx)), float(geom.get("dy_computed", dy)),
                          float(geom.get("dz_computed", dz)))
    params = params_from_config(config, nu=nu, tol=tol, max_iter=max_iter, shift_factor=shift)
    has_density = density is not None and len(density) > 0
    dens = np.ascontiguousarray(density if has_density else np.ones(nx * ny * nz), dtype=np.float32)
    bc_cm = np.ascontiguousarray(np.asarray(bc_indicator, dtype=np.float32).ravel(order="F"))  # Matrix(nNodes,3)
    f32 = np.ascontiguousarray(np.asarray(F, dtype=np.float32))
    guess = None
    if u_prev is not None and len(u_prev) == len(f32):
        guess = np.ascontiguousarray(np.asarray(u_prev, dtype=np.float32))
    u = np.empty(f32.shape[0], dtype=np.float64)
    relres = C.c_double()
    name = C.create_string_buffer(32)
    active = C.c_int64()
    st = _lib.SolveStats()
    ctx = context()
    rc = ctx.lib.hexa_solve_system(ctx.h, C.byref(grid), float(np.float32(E)), _lib.ptr(bc_cm), _lib.ptr(f32),
                                   _lib.ptr(dens), float(np.float32(min_stiffness_threshold)),
                                   int(bool(prune_voids) and has_density), int(config.get("current_outer_iter", 1)),
                                   C.byref(params), _lib.ptr(guess), _lib.ptr(u), C.byref(relres), name, 32,
                                   C.byref(st), C.byref(active))
    if rc == _lib.HEXA_ERR_CORRUPT_INPUT:
        return np.zeros(u.shape[0], dtype=np.float64), float("nan"), "Failed_Corrupt_Input"
    ctx.check(rc)
    if isinstance(stats, dict):
        stats.update(st.as_dict())
        stats["active_elements"] = int(active.value)
    return u, float(relres.value), name.value.decode()


def apply_operator(grid, factor, x, *, nu=0.3, sigma=0.0, clamp_faces=0, fixed_dof=None, ctx=None, fp32=False):
    """y = (K_ff + sigma I) x with y = 0 at fixed DOFs (one operator launch)."""
    ctx = ctx or context()
    bc = _lib.make_bc(clamp_faces, fixed_dof)
    dt = np.float32 if fp32 else np.float64
    y = np.empty(3 * (grid.nx + 1) * (grid.ny + 1) * (grid.nz + 1), dtype=dt) if isinstance(x, np.ndarray) else None
    if y is None:
        import torch
        y = torch.empty_like(x)
    fn = ctx.lib.hexa_apply_operator_f32 if fp32 else ctx.lib.hexa_apply_operator
    rc = fn(ctx.h, C.byref(grid), C.byref(bc), float(nu), _lib.ptr(factor), _lib.ptr(x), float(sigma), _lib.ptr(y))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return y


def operator_diagonal(grid, factor, *, nu=0.3, clamp_faces=0, fixed_dof=None, diag_quirk=1, ctx=None):
    ctx = ctx or context()
    bc = _lib.make_bc(clamp_faces, fixed_dof)
    d = np.empty(3 * (grid.nx + 1) * (grid.ny + 1) * (grid.nz + 1), dtype=np.float64)
    rc = ctx.lib.hexa_operator_diagonal(ctx.h, C.byref(grid), C.byref(bc), float(nu), _lib.ptr(factor),
                                        int(diag_quirk), _lib.ptr(d))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return d


def canonical_stiffness(dx=1.0, dy=1.0, dz=1.0, nu=0.3) -> np.ndarray:
    """Element.get_canonical_stiffness (24x24, E = 1)."""
    k = np.empty(576, dtype=np.float64)
    rc = _lib.load().hexa_canonical_stiffness(float(dx), float(dy), float(dz), float(nu), _lib.ptr(k))
    if rc != 0:
        raise ValueError("invalid element geometry or Poisson ratio")
    return k.reshape(24, 24, order="F")
