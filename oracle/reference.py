"""CPU restatement of the reference's FE-solve path (numpy/scipy + hexa_oracle.c):
the operator, the PCG control flow with its Jacobi and two-level multigrid
preconditioners, the filter, SIMP/OC, and the rows either side of the solve
(stress, density update, refiner transfer).

TEST INFRASTRUCTURE ONLY -- the parity checker and the timed CPU baseline.
Every function names the reference file:lines it restates (paths relative
to the reference project root).  Parity is unpinned by the reference (it has
no tests); the pins are tests/golden (exact rational element matrices) and
the first-principles checks in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .build import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        P, D, I = C.c_void_p, C.c_double, C.c_int
        L.ho_canonical_stiffness.argtypes = [D, D, D, D, I, P]
        L.ho_scalar_matrices.argtypes = [D, D, D, I, P, P]
        L.ho_apply_K.argtypes = [I, I, I, P, P, P, P]
        L.ho_diag_K.argtypes = [I, I, I, P, P, I, P]
        L.ho_element_energy.argtypes = [I, I, I, P, P, P]
        L.ho_helm_apply.argtypes = [I, I, I, P, P, P]
        L.ho_helm_rhs.argtypes = [I, I, I, P, D, P]
        L.ho_helm_extract.argtypes = [I, I, I, P, P]
        L.ho_helm_pcg.argtypes = [I, I, I, P, P, D, D, I, P, C.POINTER(D)]
        L.ho_helm_pcg.restype = I
        L.ho_cpu_matrix_free_cg.argtypes = [I, I, I, P, C.c_float, P, P, P, C.c_float, I, C.c_float, C.c_float, I, D,
                                            P, C.POINTER(D), C.POINTER(D), C.POINTER(I)]
        L.ho_cpu_matrix_free_cg.restype = I
        L.ho_num_threads.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


@dataclass(frozen=True)
class Grid:
    nx: int
    ny: int
    nz: int
    dx: float = 1.0
    dy: float = 1.0
    dz: float = 1.0

    @property
    def nnode(self):
        return (self.nx + 1) * (self.ny + 1) * (self.nz + 1)

    @property
    def nelem(self):
        return self.nx * self.ny * self.nz

    @property
    def ndof(self):
        return 3 * self.nnode


# ------------------------------------------------------------ element matrices
def canonical_stiffness(dx=1.0, dy=1.0, dz=1.0, nu=0.3, fp32=False) -> np.ndarray:
    """Element.jl:23-111 (fp32=True evaluates in Float32 as the reference)."""
    k = np.zeros(576)
    if lib().ho_canonical_stiffness(dx, dy, dz, nu, int(fp32), _p(k)) != 0:
        raise ValueError("non-positive Jacobian")
    return k.reshape(24, 24, order="F")


def scalar_matrices(dx=1.0, dy=1.0, dz=1.0, quirk=True):
    """Element.jl:113-134; quirk keeps the top face at +dz (Element.jl:116)."""
    ke, me = np.zeros(64), np.zeros(64)
    lib().ho_scalar_matrices(dx, dy, dz, int(quirk), _p(ke), _p(me))
    return ke.reshape(8, 8, order="F"), me.reshape(8, 8, order="F")


# ---------------------------------------------------------------- mesh / BCs
def element_nodes(g: Grid) -> np.ndarray:
    """0-based connectivity in n1..n8 order (src/Mesh/Mesh.jl:44-53)."""
    NX, NY = g.nx + 1, g.ny + 1
    ek, ej, ei = np.meshgrid(np.arange(g.nz), np.arange(g.ny), np.arange(g.nx), indexing="ij")
    n1 = (ei + NX * (ej + NY * ek)).ravel()
    off = [0, 1, 1 + NX, NX, NX * NY, 1 + NX * NY, 1 + NX + NX * NY, NX + NX * NY]
    return np.stack([n1 + o for o in off], axis=1)


def fixed_mask(g: Grid, clamp_faces: int = 0, fixed_dof=None) -> np.ndarray:
    NX, NY, NZ = g.nx + 1, g.ny + 1, g.nz + 1
    m = np.zeros((NZ, NY, NX, 3), dtype=bool)
    sel = [np.s_[:, :, 0], np.s_[:, :, -1], np.s_[:, 0, :], np.s_[:, -1, :], np.s_[0, :, :], np.s_[-1, :, :]]
    for b in range(6):
        if clamp_faces >> b & 1:
            m[sel[b]] = True
    m = m.reshape(-1)
    if fixed_dof is not None:
        m |= np.asarray(fixed_dof).reshape(-1) != 0
    return m


# ----------------------------------------------------------------- operators
def apply_K(g: Grid, K0, factor, x) -> np.ndarray:
    """Element scatter y = sum_e factor_e K0 u_e (GPUSolver.jl:91-128), full DOFs."""
    K0 = np.asfortranarray(K0, dtype=np.float64).ravel(order="F").copy()
    y = np.zeros(g.ndof)
    lib().ho_apply_K(g.nx, g.ny, g.nz, _p(K0), _p(np.ascontiguousarray(factor, dtype=np.float64)),
                     _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
    return y


def apply_A(g: Grid, K0, factor, x, fixed, sigma=0.0) -> np.ndarray:
    """apply_A! + shift (GPUSolver.jl:322-330,372): (K_ff + sigma I) x_free, zeros at fixed DOFs."""
    xm = np.where(fixed, 0.0, x)
    y = apply_K(g, K0, factor, xm) + sigma * xm
    y[fixed] = 0.0
    return y


def diag_K(g: Grid, K0, factor, quirk=True) -> np.ndarray:
    """compute_diagonal_atomic_kernel! (GPUSolver.jl:130-144)."""
    K0 = np.asfortranarray(K0, dtype=np.float64).ravel(order="F").copy()
    d = np.zeros(g.ndof)
    lib().ho_diag_K(g.nx, g.ny, g.nz, _p(K0), _p(np.ascontiguousarray(factor, dtype=np.float64)), int(quirk), _p(d))
    return d


def assemble_K(g: Grid, K0, factor) -> sp.csr_matrix:
    """Global COO assembly, 576 entries per element (DirectSolver.jl:62-103)."""
    en = element_nodes(g)
    dofs = (3 * en[:, :, None] + np.arange(3)[None, None, :]).reshape(g.nelem, 24)
    rows = np.repeat(dofs, 24, axis=1).ravel()
    cols = np.tile(dofs, (1, 24)).ravel()
    vals = (np.asarray(factor)[:, None] * np.asarray(K0).ravel(order="C")[None, :]).ravel()
    return sp.csr_matrix((vals, (rows, cols)), shape=(g.ndof, g.ndof))


def direct_solve(g: Grid, K0, factor, f, fixed, sigma=0.0) -> np.ndarray:
    """(K_ff + sigma I) u = f_free by sparse LU (the DirectSolver.jl method)."""
    K = assemble_K(g, K0, factor)
    free = np.nonzero(~fixed)[0]
    Kff = (K[free][:, free] + sigma * sp.identity(free.size)).tocsc()
    u = np.zeros(g.ndof)
    u[free] = spla.spsolve(Kff, np.asarray(f)[free])
    return u


# ------------------------------------------------------------ void pruning
def prune_system(nodes, elements, density, threshold, bc_indicator, F):
    """MeshPruner.prune_system (src/Mesh/MeshPruner.jl:10-87), 0-based: keeps the
    elements with density > threshold and the nodes they touch, renumbered in
    increasing old order; bc rows, loads and densities follow."""
    density = np.asarray(density, dtype=np.float32)
    active = np.nonzero(density > np.float32(threshold))[0]
    if active.size == 0:
        raise ValueError(f"MeshPruner: No active elements found (Threshold: {threshold}). System is empty.")
    n_nodes = np.asarray(nodes).shape[0]
    on = np.zeros(n_nodes, dtype=bool)
    on[np.asarray(elements)[active].ravel()] = True
    new_to_old = np.nonzero(on)[0]
    old_to_new = np.full(n_nodes, -1, dtype=np.int64)
    old_to_new[new_to_old] = np.arange(new_to_old.size)
    return dict(nodes=np.asarray(nodes)[new_to_old], elements=old_to_new[np.asarray(elements)[active]],
                bc_indicator=np.asarray(bc_indicator)[new_to_old],
                F=np.asarray(F, dtype=np.float32).reshape(-1, 3)[new_to_old].ravel(),
                density=density[active], new_to_old_node_map=new_to_old, active_element_indices=active)


def reconstruct_full_solution(u_reduced, new_to_old, n_full_nodes):
    """MeshPruner.reconstruct_full_solution (MeshPruner.jl:89-107): zeros at removed nodes."""
    u = np.zeros((n_full_nodes, 3), dtype=np.asarray(u_reduced).dtype)
    u[new_to_old] = np.asarray(u_reduced).reshape(-1, 3)
    return u.ravel()


def solve_mesh(elements, K0, factor, F, fixed, shift_factor, tol=1e-14, max_iter=100000):
    """(K_ff + sigma I) u = f_free on an arbitrary hex8 connectivity (elements:
    (nElem, 8) 0-based node indices in the K0 node order), sigma = shift_factor
    * max over free DOFs of the x-diagonal form (GPUSolver.jl:130-144, 343),
    by Jacobi-PCG on the assembled sparse matrix to a tight residual."""
    elements = np.asarray(elements)
    ndof = 3 * (int(elements.max()) + 1)
    ndof = max(ndof, np.asarray(F).size)
    dofs = (3 * elements[:, :, None] + np.arange(3)[None, None, :]).reshape(-1, 24)
    rows = np.repeat(dofs, 24, axis=1).ravel()
    cols = np.tile(dofs, (1, 24)).ravel()
    vals = (np.asarray(factor, dtype=np.float64)[:, None] * np.asarray(K0).ravel(order="C")[None, :]).ravel()
    K = sp.csr_matrix((vals, (rows, cols)), shape=(ndof, ndof))
    dq = np.zeros(ndof)
    np.add.at(dq, dofs.ravel(), np.tile(np.repeat(np.diag(K0)[0::3], 3), elements.shape[0]) *
              np.repeat(np.asarray(factor, dtype=np.float64), 24))
    free = np.nonzero(~np.asarray(fixed, dtype=bool))[0]
    sigma = shift_factor * dq[free].max() if free.size else 0.0
    A = (K[free][:, free] + sigma * sp.identity(free.size)).tocsr()
    b = np.asarray(F, dtype=np.float64)[free]
    d = A.diagonal()
    x = np.zeros_like(b)
    r = b.copy()
    nb = np.linalg.norm(b)
    u = np.zeros(ndof)
    if nb == 0.0:
        return u, sigma
    z = r / d
    p = z.copy()
    rz = r @ z
    for _ in range(max_iter):
        q = A @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.linalg.norm(r) / nb < tol:
            break
        z = r / d
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    u[free] = x
    return u, sigma


def solve_system_pruned(g: Grid, E, density, bc_indicator, F, *, min_stiffness_threshold, prune_voids,
                        current_outer_iter, shift_factor, nu=0.3, tol=1e-14):
    """Solver.solve_system's gpu path (src/Solvers/Solver.jl:39-160) with its
    pruning rule: from outer iteration 3, when fewer than 99 % of the elements
    have density > min_stiffness_threshold * 1.01f0, the MeshPruner system is
    solved and mapped back; else the full system.  factor = Float32(E .*
    density) (GPUSolver.jl:254).  Returns (U_full, active element count)."""
    nodes = np.zeros((g.nnode, 3), dtype=np.float32)
    elements = element_nodes(g)
    K0 = canonical_stiffness(g.dx, g.dy, g.dz, nu)
    density = np.asarray(density, dtype=np.float32)
    thr = np.float32(min_stiffness_threshold) * np.float32(1.01)
    prune = bool(prune_voids) and current_outer_iter >= 3
    if prune:
        prune = np.count_nonzero(density > thr) < g.nelem * 0.99
    if not prune:
        fixed = np.asarray(bc_indicator).reshape(-1) > 0
        fac = (np.float32(E) * density).astype(np.float64)
        u, _ = solve_mesh(elements, K0, fac, F, fixed, shift_factor, tol)
        return u, g.nelem
    P = prune_system(nodes, elements, density, thr, bc_indicator, F)
    fixed = np.asarray(P["bc_indicator"]).reshape(-1) > 0
    fac = (np.float32(E) * P["density"]).astype(np.float64)
    u_red, _ = solve_mesh(P["elements"], K0, fac, P["F"], fixed, shift_factor, tol)
    return reconstruct_full_solution(u_red, P["new_to_old_node_map"], g.nnode), int(P["active_element_indices"].size)


# ----------------------------------------------------- reference PCG control
@dataclass
class PcgInfo:
    iterations: list
    shifts: list
    final_rel: float
    success: bool
    name: str


class ReferenceMG:
    """The reference's two-level additive preconditioner, restated in numpy:
    setup_multigrid and apply_mg_vcycle! (GPUGeometricMultigrid.jl:252-346)
    with the restriction / prolongation kernels (:60-204), in Float32 as the
    reference's workspace.  z = D^-1 r (fine Jacobi) + P (r_c ./ (D_c + 1e-9)),
    r_c = P^T r: P interpolates trilinearly from the nodes of a grid of
    max(1, n/2) elements per axis (element size 2h) at the fine nodes'
    coordinates, D_c is 1 plus the x-diagonal of the unit-modulus coarse K0
    (nu fixed at 0.3) summed over the coarse elements that hold a fine node
    (modulus 1, the rest 0.001).  Atomic sums run in a fixed order here."""

    def __init__(self, g: Grid, free):
        f32 = np.float32
        self.g, self.free = g, np.asarray(free)
        nxc, nyc, nzc = max(1, g.nx // 2), max(1, g.ny // 2), max(1, g.nz // 2)
        self.nc = (nxc, nyc, nzc)
        hc = [f32(f32(h) * f32(2.0)) for h in (g.dx, g.dy, g.dz)]
        NX, NY, NZ = g.nx + 1, g.ny + 1, g.nz + 1
        k, j, i = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
        # node coordinates (i-1)*dx in Float32 (Mesh.jl:36), normalised by the coarse size (:206-214)
        coords = [(a.ravel().astype(f32) * f32(h)) / hcc for a, h, hcc in zip((i, j, k), (g.dx, g.dy, g.dz), hc)]
        lo = [np.floor(c).astype(np.int64) for c in coords]
        t = [(c - l.astype(f32)).astype(f32) for c, l in zip(coords, lo)]
        one = f32(1.0)
        self.corners = []
        for dk in (0, 1):
            for dj in (0, 1):
                for di in (0, 1):
                    ci, cj, ck = lo[0] + di, lo[1] + dj, lo[2] + dk
                    wx = t[0] if di else one - t[0]
                    wy = t[1] if dj else one - t[1]
                    wz = t[2] if dk else one - t[2]
                    w = ((wx * wy) * wz).astype(f32)
                    ok = (ci >= 0) & (cj >= 0) & (ck >= 0) & (ci <= nxc) & (cj <= nyc) & (ck <= nzc)
                    self.corners.append((np.nonzero(ok)[0], (ci + cj * (nxc + 1) + ck * (nxc + 1) * (nyc + 1))[ok],
                                         w[ok]))
        # corner order of the kernels: (0,0,0) (1,0,0) (0,1,0) (1,1,0) (0,0,1) (1,0,1) (0,1,1) (1,1,1)
        # coarse modulus: 1 where a fine node's floor lands inside, else 0.001 (:218-229)
        ex, ey, ez = lo
        inside = (ex >= 0) & (ey >= 0) & (ez >= 0) & (ex < nxc) & (ey < nyc) & (ez < nzc)
        rho_c = np.full(nxc * nyc * nzc, f32(0.001))
        rho_c[(ex + ey * nxc + ez * nxc * nyc)[inside]] = f32(1.0)
        kd = np.diag(canonical_stiffness(float(hc[0]), float(hc[1]), float(hc[2]), 0.3, fp32=True)).astype(f32)
        gc = Grid(nxc, nyc, nzc)
        en = element_nodes(gc)
        self.nnc = gc.nnode
        Dc = np.ones(3 * gc.nnode, f32)  # fill!(diag_coarse, 1.0f0), then the atomic adds (:47-58)
        for a in range(8):
            kv = (kd[3 * a] * rho_c).astype(f32)
            for c in range(3):
                np.add.at(Dc, 3 * en[:, a] + c, kv)
        self.Dc = Dc

    def apply(self, r_free, Minv):
        f32 = np.float32
        z = r_free * Minv
        rf = np.zeros(self.g.ndof, f32)
        rf[self.free] = np.asarray(r_free).astype(f32)
        rc = np.zeros(3 * self.nnc, f32)
        for nodes, cidx, w in self.corners:
            for c in range(3):
                np.add.at(rc, 3 * cidx + c, (rf[3 * nodes + c] * w).astype(f32))
        xc = (rc / (self.Dc + f32(1e-9))).astype(f32)
        zf = np.zeros(self.g.ndof, f32)
        for nodes, cidx, w in self.corners:
            for c in range(3):
                zf[3 * nodes + c] = (zf[3 * nodes + c] + (xc[3 * cidx + c] * w).astype(f32)).astype(f32)
        return z + zf[self.free].astype(np.float64)


def pcg_reference(g: Grid, K0, factor, f, fixed, *, tol, max_iter, shift_factor, stagnation_tol=0.0,
                  max_shift_attempts=3, shift_multiplier=10.0, u_guess=None, diag_quirk=True, cadence=10,
                  precond="jacobi"):
    """gpu_matrix_free_cg_solve (GPUSolver.jl:182-465) on the free DOFs, FP64:
    shift attempts, the NaN/divergence tests, stagnation acceptance, the
    best-iterate return and, with precond="multigrid", the reference's
    two-level preconditioner (ReferenceMG) with its fall-back to Jacobi on a
    NaN or divergence (:389-437).  Returns (u, final relres, PcgInfo)."""
    free = ~fixed
    d = diag_K(g, K0, factor, quirk=diag_quirk)[free]
    max_diag = d.max()
    if np.isnan(max_diag) or np.isinf(max_diag):
        return np.zeros(g.ndof), float("nan"), PcgInfo([], [], float("nan"), False, "Failed_Corrupt_Input")
    b = np.asarray(f, dtype=np.float64)[free]
    norm_b = np.linalg.norm(b)
    n = b.size

    def A(v):
        full = np.zeros(g.ndof)
        full[free] = v
        return apply_K(g, K0, factor, full)[free]

    want_mg = precond == "multigrid"
    mg = ReferenceMG(g, free) if want_mg else None
    use_mg = want_mg
    x = np.zeros(n)
    best_x = np.zeros(n)
    final_rel = 0.0
    success = False
    iters, shifts = [], []
    while True:
        cur_shift = shift_factor
        fallback = False
        for attempt in range(1, max_shift_attempts + 1):
            real_shift = cur_shift * max_diag
            shifts.append(real_shift)
            diverged = False
            if u_guess is not None and attempt == 1 and use_mg == want_mg:
                x = np.asarray(u_guess, dtype=np.float64)[free].copy()
            elif attempt > 1 or use_mg != want_mg:
                x = np.zeros(n)
            Minv = 1.0 / (d + real_shift)
            M = (lambda v: mg.apply(v, Minv)) if use_mg else (lambda v: v * Minv)
            r = b - (A(x) + real_shift * x)
            z = M(r)
            p = z.copy()
            rz = r @ z
            best_rel = np.inf
            solve_ok = False
            k = 0
            for k in range(1, max_iter + 1):
                Ap = A(p) + real_shift * p
                denom = p @ Ap
                if abs(denom) < 1e-20:
                    break
                alpha = rz / denom
                x = x + alpha * p
                r = r - alpha * Ap
                if k == 1 or (cadence <= 1) or k % cadence == 0:
                    rel = np.linalg.norm(r) / norm_b
                    final_rel = rel
                    if rel < best_rel:
                        best_rel = rel
                        best_x = x.copy()
                    if rel < tol:
                        solve_ok = True
                        break
                    if np.isnan(rel) or np.isinf(rel) or rel > 10.0 or (k > 500 and rel > best_rel * 100.0):
                        if use_mg:
                            fallback = True
                        else:
                            diverged = True
                        break
                z = M(r)
                rz_new = r @ z
                p = z + (rz_new / rz) * p
                rz = rz_new
            iters.append(k)
            if fallback:
                break
            if solve_ok:
                success = True
                break
            if diverged and attempt < max_shift_attempts:
                cur_shift *= shift_multiplier
                continue
            if stagnation_tol > 0.0 and best_rel < stagnation_tol:
                success = True
                x = best_x
                break
            cur_shift *= shift_multiplier
        if fallback:  # restart every attempt with the Jacobi preconditioner
            use_mg = False
            continue
        break
    if not success:
        x = best_x
    u = np.zeros(g.ndof)
    u[free] = x
    return u, final_rel, PcgInfo(iters, shifts, final_rel, success, "GMG_GPU" if use_mg else "Jacobi_GPU")


def cg_tight(g: Grid, K0, factor, f, fixed, sigma=0.0, tol=1e-13, max_iter=200000, x0=None):
    """Plain Jacobi-PCG to a tight relative residual (oracle solution for grids too big for LU).

    x0 (full DOF vector) only shortens the run: the iteration stops on this
    operator's own residual ||b - A x|| / ||b|| < tol, so the answer is the
    oracle's whatever the start."""
    free = ~fixed
    d = diag_K(g, K0, factor, quirk=False)[free] + sigma
    b = np.asarray(f, dtype=np.float64)[free]

    def A(v):
        full = np.zeros(g.ndof)
        full[free] = v
        return apply_K(g, K0, factor, full)[free] + sigma * v

    x = np.zeros_like(b) if x0 is None else np.asarray(x0, dtype=np.float64)[free].copy()
    r = b - A(x) if x0 is not None else b.copy()
    z = r / d
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for k in range(max_iter):
        Ap = A(p)
        a = rz / (p @ Ap)
        x += a * p
        r -= a * Ap
        if np.linalg.norm(r) / nb < tol:
            break
        z = r / d
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    r = b - A(x)
    u = np.zeros(g.ndof)
    u[free] = x
    return u, np.linalg.norm(r) / nb, k + 1


# --------------------------------------------------------------- Helmholtz
def helm_matrix(g: Grid, R: float, quirk=True):
    Ke, Me = scalar_matrices(g.dx, g.dy, g.dz, quirk)
    return R * R * Ke + Me


def helm_apply(g: Grid, Ae, x):
    y = np.zeros(g.nnode)
    A = np.asfortranarray(Ae).ravel(order="F").copy()
    lib().ho_helm_apply(g.nx, g.ny, g.nz, _p(A), _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
    return y


def helm_rhs(g: Grid, rho):
    b = np.zeros(g.nnode)
    lib().ho_helm_rhs(g.nx, g.ny, g.nz, _p(np.ascontiguousarray(rho, dtype=np.float64)), g.dx * g.dy * g.dz / 8.0, _p(b))
    return b


def helm_extract(g: Grid, psi):
    out = np.zeros(g.nelem)
    lib().ho_helm_extract(g.nx, g.ny, g.nz, _p(np.ascontiguousarray(psi, dtype=np.float64)), _p(out))
    return out


def helmholtz_reference(g: Grid, rho, R, tol, max_iter=200, quirk=True):
    """solve_helmholtz_on_gpu (GPUHelmholtz.jl:190-266): Jacobi-PCG, test every 10 iterations."""
    Ae = helm_matrix(g, R, quirk)
    en = element_nodes(g)
    diag = np.zeros(g.nnode)
    np.add.at(diag, en.ravel(), np.tile(np.diag(Ae), g.nelem))
    inv_diag = 1.0 / diag
    b = helm_rhs(g, rho)
    norm_b = np.linalg.norm(b)
    if norm_b == 0.0:
        return np.asarray(rho, dtype=np.float64).copy(), 0, 0.0
    x = np.zeros(g.nnode)
    r = b.copy()
    z = r * inv_diag
    p = z.copy()
    rho_old = r @ z
    final_rel, final_iter = 0.0, 0
    for it in range(1, max_iter + 1):
        final_iter = it
        Ap = helm_apply(g, Ae, p)
        alpha = rho_old / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        if it % 10 == 0:
            final_rel = np.linalg.norm(r) / norm_b
            if final_rel < tol:
                break
        z = r * inv_diag
        rho_new = r @ z
        p = z + (rho_new / rho_old) * p
        rho_old = rho_new
    return helm_extract(g, x), final_iter, final_rel


def helmholtz_pcg_c(g: Grid, rho, R, tol, max_iter=200, quirk=True):
    """helmholtz_reference in C with OpenMP (oracle/hexa_oracle.c ho_helm_pcg):
    the same Jacobi-PCG loop, for grids where the numpy loop is too slow."""
    A = np.asfortranarray(helm_matrix(g, R, quirk)).ravel(order="F").copy()
    out = np.empty(g.nelem)
    rel = C.c_double()
    it = lib().ho_helm_pcg(g.nx, g.ny, g.nz, _p(A), _p(np.ascontiguousarray(rho, dtype=np.float64)),
                           g.dx * g.dy * g.dz / 8.0, float(tol), int(max_iter), _p(out), C.byref(rel))
    if it < 0:
        raise MemoryError("ho_helm_pcg: allocation failed")
    return out, it, rel.value


_HELM_LU = {}


def helmholtz_direct(g: Grid, rho, R, quirk=True, shift=0.0):
    """assemble_helmholtz_system + apply_helmholtz_filter_cpu (TopOpt.jl:32-127);
    the reference's CPU path adds a 1e-9 diagonal shift (TopOpt.jl:75-76).  The
    sparse LU of the (constant) filter matrix is cached per grid and radius."""
    key = (g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, float(R), bool(quirk), float(shift))
    lu = _HELM_LU.get(key)
    if lu is None:
        Ae = helm_matrix(g, R, quirk)
        en = element_nodes(g)
        rows = np.repeat(en, 8, axis=1).ravel()
        cols = np.tile(en, (1, 8)).ravel()
        vals = np.tile(Ae.ravel(order="C"), g.nelem)
        A = sp.csc_matrix((vals, (rows, cols)), shape=(g.nnode, g.nnode))
        if shift:
            A = A + shift * sp.identity(g.nnode, format="csc")
        lu = spla.splu(A.tocsc())
        if len(_HELM_LU) > 8:
            _HELM_LU.clear()
        _HELM_LU[key] = lu
    psi = lu.solve(helm_rhs(g, rho))
    return helm_extract(g, psi)


# -------------------------------------------------------------- SIMP / OC
def simp_factors(rho, Emin=1e-9, E0=1.0, penal=3.0):
    return Emin + np.power(rho, penal) * (E0 - Emin)


def element_energy(g: Grid, K0, u):
    ce = np.zeros(g.nelem)
    K = np.asfortranarray(K0).ravel(order="F").copy()
    lib().ho_element_energy(g.nx, g.ny, g.nz, _p(K), _p(np.ascontiguousarray(u, dtype=np.float64)), _p(ce))
    return ce


def sensitivities(g: Grid, K0, rho, u, Emin=1e-9, E0=1.0, penal=3.0):
    ce = element_energy(g, K0, u)
    dc = -penal * np.power(rho, penal - 1.0) * (E0 - Emin) * ce
    c = float(np.sum(simp_factors(rho, Emin, E0, penal) * ce))
    return dc, c


def oc_update(x, dc, dv, volfrac, move=0.2, tol=1e-12):
    """OC step of the 88-line code (Andreassen et al. 2011): bisection on lambda
    in [0, 1e9] until (l2-l1)/(l1+l2) <= tol; returns the update at the last
    midpoint tested and that midpoint."""
    l1, l2 = 0.0, 1e9
    n = x.size
    xnew, lmid = x, 0.5 * (l1 + l2)
    while (l2 - l1) / (l1 + l2) > tol:
        lmid = 0.5 * (l2 + l1)
        xnew = np.maximum(0.0, np.maximum(x - move, np.minimum(1.0, np.minimum(x + move, x * np.sqrt(-dc / dv / lmid)))))
        if xnew.sum() > volfrac * n:
            l1 = lmid
        else:
            l2 = lmid
    return xnew, lmid


def simp_loop(g: Grid, x0, f, fixed, *, nu=0.3, Emin=1e-9, E0=1.0, penal=3.0, volfrac=0.3, R=0.6, move=0.2,
              n_iter=10, sigma_factor=1e-10, solve_tol=1e-13, start=None):
    """The SIMP + OC loop of topopt.run_simp, with exact (LU) filters and tight solves.

    start(i) may return a starting vector for iteration i's CG on grids too big
    for LU; it changes the run time only (see cg_tight)."""
    K0 = canonical_stiffness(g.dx, g.dy, g.dz, nu)
    dv = helmholtz_direct(g, np.ones(g.nelem), R, quirk=False)
    x = np.asarray(x0, dtype=np.float64).copy()
    hist = []
    for _ in range(n_iter):
        xphys = helmholtz_direct(g, x, R, quirk=False)
        fac = simp_factors(xphys, Emin, E0, penal)
        sigma = sigma_factor * diag_K(g, K0, fac, quirk=True)[~fixed].max()
        if g.ndof <= 60000:
            u = direct_solve(g, K0, fac, f, fixed, sigma)
        else:
            u, _, _ = cg_tight(g, K0, fac, f, fixed, sigma, tol=solve_tol,
                               x0=start(len(hist)) if start else None)
        dc, c = sensitivities(g, K0, xphys, u, Emin, E0, penal)
        dcx = helmholtz_direct(g, dc, R, quirk=False)
        hist.append(dict(compliance=c, u=u, dc=dc, xphys=xphys))
        x, _ = oc_update(x, dcx, dv, volfrac, move)
    return hist


# ------------------------------------------------------------ CPU baseline
def cpu_matrix_free_cg(g: Grid, E, density, f, fixed_dof, *, nu=0.3, min_stiffness_threshold=1e-3, max_iter=1000,
                       tol=1e-6, shift_factor=1e-6, nthreads=None, max_seconds=0.0):
    """CPUSolver.solve_system_cpu (CPUSolver.jl:56-272) in Float32, timed.

    Returns (u Float32, relres, iterations, seconds)."""
    L = lib()
    K0 = canonical_stiffness(g.dx, g.dy, g.dz, nu, fp32=True).astype(np.float32).ravel(order="F").copy()
    x = np.zeros(g.ndof, dtype=np.float32)
    rel, sec, it = C.c_double(), C.c_double(), C.c_int()
    nthreads = nthreads or L.ho_num_threads()
    L.ho_cpu_matrix_free_cg(g.nx, g.ny, g.nz, _p(K0), float(E), _p(np.ascontiguousarray(density, dtype=np.float32)),
                            _p(np.ascontiguousarray(f, dtype=np.float32)),
                            _p(np.ascontiguousarray(fixed_dof, dtype=np.uint8)), float(min_stiffness_threshold),
                            int(max_iter), float(tol), float(shift_factor), int(nthreads), float(max_seconds), _p(x),
                            C.byref(rel), C.byref(sec), C.byref(it))
    return x, rel.value, it.value, sec.value


def num_threads() -> int:
    return int(lib().ho_num_threads())


def wall(fn, *a, **k):
    t = time.perf_counter()
    r = fn(*a, **k)
    return r, time.perf_counter() - t


# ------------------------------------------------------------------- stress
def _jacobi_rotate(spp, sqq, spq, spr, sqr, v, p, q):
    """One rotation of Stress.jl:89-140 on arrays of elements (float32), in place."""
    f32 = np.float32
    h = spq.copy()
    g = f32(100.0) * np.abs(h)
    act = (np.abs(spp) + g != np.abs(spp)) | (np.abs(sqq) + g != np.abs(sqq))
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):  # inactive lanes; the GPU overflows alike
        theta = f32(0.5) * (sqq - spp) / h
        t = f32(1.0) / (np.abs(theta) + np.sqrt(theta * theta + f32(1.0)))
    t = np.where(theta < 0, -t, t).astype(f32)
    c = (f32(1.0) / np.sqrt(t * t + f32(1.0))).astype(f32)
    s = (t * c).astype(f32)
    tau = (s / (f32(1.0) + c)).astype(f32)
    spp_n = spp - t * spq
    sqq_n = sqq + t * spq
    tmp = spr.copy()
    spr_n = spr - s * (sqr + tau * spr)
    sqr_n = sqr + s * (tmp - tau * sqr)
    for arr, new in ((spp, spp_n), (sqq, sqq_n), (spr, spr_n), (sqr, sqr_n)):
        arr[act] = new[act]
    spq[act] = 0.0
    for r in range(3):
        vp = v[r][p].copy()
        vp_n = vp - s * (v[r][q] + tau * vp)
        vq_n = v[r][q] + s * (vp - tau * v[r][q])
        v[r][p][act] = vp_n[act]
        v[r][q][act] = vq_n[act]


def eigen3x3(sxx, syy, szz, sxy, syz, sxz):
    """eigen3x3_device (Stress.jl:95-157) on arrays of symmetric tensors,
    Float32: at most 12 sweeps of the (1,2), (1,3), (2,3) Jacobi rotations,
    stopped per tensor once every off-diagonal is below 1e-9, then sorted
    descending.  Returns (eigenvalues (n, 3), direction of the largest (n, 3),
    direction of the smallest (n, 3))."""
    f32 = np.float32
    n = np.asarray(sxx).size
    s11, s22, s33, s12, s23, s13 = (np.asarray(a, dtype=f32).reshape(-1).copy() for a in (sxx, syy, szz, sxy, syz, sxz))
    v = [[np.full(n, f32(1.0 if r == c else 0.0)) for c in range(3)] for r in range(3)]
    done = np.zeros(n, bool)
    for _ in range(12):
        done |= np.maximum(np.abs(s12), np.maximum(np.abs(s23), np.abs(s13))) < f32(1e-9)
        live = ~done
        if not live.any():
            break
        sub = [a[live] for a in (s11, s22, s33, s12, s23, s13)]
        vs = [[v[r][c][live] for c in range(3)] for r in range(3)]
        a11, a22, a33, a12, a23, a13 = sub
        _jacobi_rotate(a11, a22, a12, a13, a23, vs, 0, 1)
        _jacobi_rotate(a11, a33, a13, a12, a23, vs, 0, 2)
        _jacobi_rotate(a22, a33, a23, a12, a13, vs, 1, 2)
        for arr, new in zip((s11, s22, s33, s12, s23, s13), (a11, a22, a33, a12, a23, a13)):
            arr[live] = new
        for r in range(3):
            for c in range(3):
                v[r][c][live] = vs[r][c]

    def swap(ma, mb, ca, cb):
        m = ma < mb
        ta = ma.copy()
        ma[m] = mb[m]
        mb[m] = ta[m]
        for r in range(3):
            t = v[r][ca].copy()
            v[r][ca][m] = v[r][cb][m]
            v[r][cb][m] = t[m]
    swap(s11, s22, 0, 1)
    swap(s22, s33, 1, 2)
    swap(s11, s22, 0, 1)
    principal = np.stack([s11, s22, s33], axis=1)
    dmax = np.stack([v[0][0], v[1][0], v[2][0]], axis=1)
    dmin = np.stack([v[0][2], v[1][2], v[2][2]], axis=1)
    return principal, dmax, dmin


def stress_field(g: Grid, u, density, E, nu):
    """Stress.stress_kernel! (Stress.jl:159-285) restated in numpy, Float32, all
    elements at once: centre-point strain/stress with E_loc = E*density, von
    Mises, principal stresses by 12 cyclic Jacobi sweeps (sorted descending),
    directions of the largest/smallest, L1 norm, Voigt stress.  Element-major
    arrays (principal[e, i])."""
    f32 = np.float32
    ne = g.nelem
    e = np.arange(ne)
    i = e % g.nx
    j = (e // g.nx) % g.ny
    k = e // (g.nx * g.ny)
    NX, NY = g.nx + 1, g.ny + 1
    dens = np.asarray(density, dtype=f32)
    uf = np.asarray(u).astype(f32)
    DI = [0, 1, 1, 0, 0, 1, 1, 0]
    DJ = [0, 0, 1, 1, 0, 0, 1, 1]
    DK = [0, 0, 0, 0, 1, 1, 1, 1]
    dx, dy, dz = f32(g.dx), f32(g.dy), f32(g.dz)
    J = [[np.zeros(ne, f32) for _ in range(3)] for _ in range(3)]
    for a in range(8):
        x = (i + DI[a]).astype(f32) * dx
        y = (j + DJ[a]).astype(f32) * dy
        z = (k + DK[a]).astype(f32) * dz
        w = [f32(0.125) if DI[a] else f32(-0.125), f32(0.125) if DJ[a] else f32(-0.125),
             f32(0.125) if DK[a] else f32(-0.125)]
        for r in range(3):
            J[r][0] += w[r] * x
            J[r][1] += w[r] * y
            J[r][2] += w[r] * z
    (j11, j12, j13), (j21, j22, j23), (j31, j32, j33) = J
    det = j11 * (j22 * j33 - j23 * j32) - j12 * (j21 * j33 - j23 * j31) + j13 * (j21 * j32 - j22 * j31)
    det = np.where(det <= f32(1e-12), f32(1.0), det).astype(f32)
    idt = f32(1.0) / det
    A = [[(j22 * j33 - j23 * j32) * idt, -(j12 * j33 - j13 * j32) * idt, (j12 * j23 - j13 * j22) * idt],
         [-(j21 * j33 - j23 * j31) * idt, (j11 * j33 - j13 * j31) * idt, -(j11 * j23 - j13 * j21) * idt],
         [(j21 * j32 - j22 * j31) * idt, -(j11 * j32 - j12 * j31) * idt, (j11 * j22 - j12 * j21) * idt]]
    exx, eyy, ezz, gxy, gyz, gxz = (np.zeros(ne, f32) for _ in range(6))
    for a in range(8):
        n = (i + DI[a]) + NX * ((j + DJ[a]) + NY * (k + DK[a]))
        ux, uy, uz = uf[3 * n], uf[3 * n + 1], uf[3 * n + 2]
        w = [f32(0.125) if DI[a] else f32(-0.125), f32(0.125) if DJ[a] else f32(-0.125),
             f32(0.125) if DK[a] else f32(-0.125)]
        ddx = w[0] * A[0][0] + w[1] * A[1][0] + w[2] * A[2][0]
        ddy = w[0] * A[0][1] + w[1] * A[1][1] + w[2] * A[2][1]
        ddz = w[0] * A[0][2] + w[1] * A[1][2] + w[2] * A[2][2]
        exx += ddx * ux
        eyy += ddy * uy
        ezz += ddz * uz
        gxy += ddy * ux + ddx * uy
        gyz += ddz * uy + ddy * uz
        gxz += ddz * ux + ddx * uz
    E, nu = f32(E), f32(nu)
    fact = (E * dens) / ((f32(1.0) + nu) * (f32(1.0) - f32(2.0) * nu))
    c1, c2, c3 = (f32(1.0) - nu) * fact, nu * fact, (f32(0.5) - nu) * fact
    sxx = c1 * exx + c2 * eyy + c2 * ezz
    syy = c2 * exx + c1 * eyy + c2 * ezz
    szz = c2 * exx + c2 * eyy + c1 * ezz
    sxy, syz, sxz = c3 * gxy, c3 * gyz, c3 * gxz
    voigt = np.stack([sxx, syy, szz, sxy, syz, sxz], axis=1)
    vm = np.sqrt(np.maximum(f32(0.0), f32(0.5) * ((sxx - syy) ** 2 + (syy - szz) ** 2 + (szz - sxx) ** 2)
                            + f32(3.0) * (sxy ** 2 + syz ** 2 + sxz ** 2)))
    principal, dmax, dmin = eigen3x3(sxx, syy, szz, sxy, syz, sxz)
    s11, s22, s33 = principal[:, 0], principal[:, 1], principal[:, 2]
    l1 = np.abs(s11) + np.abs(s22) + np.abs(s33)
    zero = dens < f32(1e-6)
    for arr in (principal, dmax, dmin, voigt):
        arr[zero] = 0.0
    for arr in (vm, l1):
        arr[zero] = 0.0
    return dict(principal=principal, vonmises=vm.astype(f32), voigt=voigt.astype(f32), l1=l1.astype(f32),
                dir_max=dmax, dir_min=dmin)


# -------------------------------------------------------------- refinement
def remap_fields(old, new_dims, new_h, lengths, density, alpha=None, projection=True):
    """MeshRefiner.jl:188-240 restated in numpy (Float32): trilinear transfer
    of the cell-centred density to the new grid's centroids, projected in the
    "hard" update, and the lower-corner cell's alpha."""
    f32 = np.float32
    onx, ony, onz = old
    nnx, nny, nnz = new_dims
    e = np.arange(nnx * nny * nnz, dtype=np.int64)
    ix = e % nnx + 1
    iy = (e // nnx) % nny + 1
    iz = e // (nnx * nny) + 1
    cx = (ix.astype(f32) - f32(0.5)) * f32(new_h[0])
    cy = (iy.astype(f32) - f32(0.5)) * f32(new_h[1])
    cz = (iz.astype(f32) - f32(0.5)) * f32(new_h[2])
    u = np.clip((cx / f32(lengths[0])) * f32(onx), f32(0.5), f32(onx) - f32(0.5)).astype(f32)
    v = np.clip((cy / f32(lengths[1])) * f32(ony), f32(0.5), f32(ony) - f32(0.5)).astype(f32)
    w = np.clip((cz / f32(lengths[2])) * f32(onz), f32(0.5), f32(onz) - f32(0.5)).astype(f32)
    u0 = np.floor(u - f32(0.5)).astype(np.int64)
    v0 = np.floor(v - f32(0.5)).astype(np.int64)
    w0 = np.floor(w - f32(0.5)).astype(np.int64)
    tx = np.clip((u - f32(0.5)) - u0.astype(f32), 0, 1).astype(f32)
    ty = np.clip((v - f32(0.5)) - v0.astype(f32), 0, 1).astype(f32)
    tz = np.clip((w - f32(0.5)) - w0.astype(f32), 0, 1).astype(f32)
    i0, i1 = np.clip(u0, 0, onx - 1), np.clip(u0 + 1, 0, onx - 1)
    j0, j1 = np.clip(v0, 0, ony - 1), np.clip(v0 + 1, 0, ony - 1)
    k0, k1 = np.clip(w0, 0, onz - 1), np.clip(w0 + 1, 0, onz - 1)
    d = np.asarray(density, dtype=f32)

    def at(i, j, k):
        return d[i + onx * j + onx * ony * k]
    one = f32(1.0)
    c00 = at(i0, j0, k0) * (one - tx) + at(i1, j0, k0) * tx
    c10 = at(i0, j1, k0) * (one - tx) + at(i1, j1, k0) * tx
    c01 = at(i0, j0, k1) * (one - tx) + at(i1, j0, k1) * tx
    c11 = at(i0, j1, k1) * (one - tx) + at(i1, j1, k1) * tx
    c0 = c00 * (one - ty) + c10 * ty
    c1 = c01 * (one - ty) + c11 * ty
    val = (c0 * (one - tz) + c1 * tz).astype(f32)
    raw = val.copy()
    if projection:
        val = np.where(val > f32(0.4), f32(1.0), np.where(val < f32(0.2), f32(0.0001), val)).astype(f32)
    na = None if alpha is None else np.asarray(alpha, dtype=f32)[i0 + onx * j0 + onx * ony * k0]
    return val, na, raw


def remap_displacement(old, new, u):
    """Trilinear transfer of nodal xyz displacements from grid `old` to grid
    `new` (element counts per axis, same box): new node i sits at old node
    coordinate i * old_n / new_n.  No reference counterpart (the reference
    restarts from zero after a refinement, Main.jl:412-413)."""
    onx, ony, onz = old
    nnx, nny, nnz = new
    U = np.asarray(u, dtype=np.float64).reshape(onz + 1, ony + 1, onx + 1, 3)

    def axis(nn, on):
        s = np.clip(np.arange(nn + 1) * on / nn, 0.0, on)  # (i * on) / nn, as the kernel
        i0 = np.clip(np.floor(s).astype(np.int64), 0, on - 1)
        return i0, s - i0
    i0, tx = axis(nnx, onx)
    j0, ty = axis(nny, ony)
    k0, tz = axis(nnz, onz)
    K, J, I = np.meshgrid(np.arange(nnz + 1), np.arange(nny + 1), np.arange(nnx + 1), indexing="ij")
    a, b, c = i0[I], j0[J], k0[K]
    x, y, z = tx[I][..., None], ty[J][..., None], tz[K][..., None]
    out = ((U[c, b, a] * (1 - x) + U[c, b, a + 1] * x) * (1 - y) +
           (U[c, b + 1, a] * (1 - x) + U[c, b + 1, a + 1] * x) * y) * (1 - z) + \
          ((U[c + 1, b, a] * (1 - x) + U[c + 1, b, a + 1] * x) * (1 - y) +
           (U[c + 1, b + 1, a] * (1 - x) + U[c + 1, b + 1, a + 1] * x) * y) * z
    return out.reshape(-1)


# ---------------------------------------------------------- density update
def density_filter_radius(p, dx, dy, dz):
    """The radius schedule of TopOpt.jl:265-298 in Float32: (R_length, R_effective)."""
    f32 = np.float32
    interm_frac = f32(p["filter_R_interm_iter_perc"]) / f32(100.0)
    dim = f32(p["max_domain_dim"])
    r_init = f32(p["filter_R_init_perc"]) / f32(100.0) * dim
    r_interm = f32(p["filter_R_interm_perc"]) / f32(100.0) * dim
    r_final = f32(p["filter_R_final_perc"]) / f32(100.0) * dim
    n = int(p["number_of_iterations"])
    interm = max(1, int(np.rint(interm_frac * f32(n))))  # Julia's round: ties to even
    calc = min(int(p["iter"]), n)
    if calc <= interm:
        t = f32(calc - 1) / f32(interm - 1) if interm > 1 else f32(0.0)
        r = r_init * (f32(1.0) - t) + r_interm * t
    else:
        t = f32(calc - interm) / f32(n - interm) if n > interm else f32(0.0)
        r = r_interm * (f32(1.0) - t) + r_final * t
    safe = f32(p["minimum_filter_radius_as_elements"]) * ((f32(dx) + f32(dy) + f32(dz)) / f32(3.0))
    r = safe if r < safe else r
    return f32(r), f32(r) / f32(2.5)


def update_density(density, l1, protected, original, p, h, filter_fn=None):
    """TopologyOptimization.update_density! (TopOpt.jl:211-482) restated in
    numpy Float32.  p holds the scalars update_density! reads (the field
    names of hexa_density_update_params); h = (dx, dy, dz); filter_fn(proposal,
    R_effective) stands for the GPU filter (None: no filter).  Returns the
    new density and the statistics; the change sum is taken in FP64 and
    rounded once (the reference's Float32 chunk sums depend on its thread
    count)."""
    f32 = np.float32
    dens = np.asarray(density, dtype=f32)
    l1 = np.asarray(l1, dtype=f32)
    orig = np.asarray(original, dtype=f32)
    prot = np.zeros(dens.size, bool) if protected is None else np.asarray(protected).astype(bool)
    free = ~prot
    stats = dict(status=0, filter_used=0, filter_nan_fallback=0, mean_change=f32(0), R_length=f32(0),
                 current_threshold=f32(0), R_effective=f32(0), active_count=0, candidates=0, culled=0)
    if np.isnan(l1).any():  # TopOpt.jl:230-236
        stats["status"] = 1
        return dens.copy(), stats
    min_d, max_d = f32(p["min_density"]), f32(p["max_density"])
    with np.errstate(over="ignore", invalid="ignore"):
        val = (l1 / f32(p["l1_stress_allowable"])) / f32(p["E"])
    prop = np.where(prot, orig, np.maximum(val, min_d)).astype(f32)  # TopOpt.jl:254-263
    R, Reff = density_filter_radius(p, *h)
    stats["R_length"], stats["R_effective"] = R, Reff
    filt = prop
    if float(Reff) > 1e-4 and filter_fn is not None:
        stats["filter_used"] = 1
        filt = np.asarray(filter_fn(prop, Reff), dtype=f32)
        if np.isnan(filt).any():  # TopOpt.jl:360-363
            stats["filter_nan_fallback"] = 1
            filt = prop
    new = dens.copy()
    with np.errstate(invalid="ignore"):
        raw = np.maximum(filt, min_d)
        eff = np.minimum(raw, max_d)
        diff = np.abs(eff - dens)  # TopOpt.jl:376-393
    change = float(diff[free].astype(np.float64).sum())
    act1 = int(np.count_nonzero(raw[free] > min_d))
    stats["mean_change"] = f32(f32(change) / f32(act1)) if act1 > 0 else f32(0)
    new[free] = raw[free]
    it, n = int(p["iter"]), int(p["number_of_iterations"])  # TopOpt.jl:420-428
    if it > n:
        thr = f32(p["final_density_threshold"])
    else:
        thr = f32(p["final_density_threshold"]) * f32(min(max(f32(it) / f32(n), f32(0)), f32(1)))
    stats["current_threshold"] = f32(thr)
    new[free] = np.minimum(new[free], max_d)  # TopOpt.jl:430-447
    live = free & (new > min_d)
    active = int(np.count_nonzero(live)) + int(np.count_nonzero(prot & (orig > min_d)))
    cands = np.nonzero(live & (new < thr))[0]
    allowed = int(np.floor(f32(active) * f32(p["max_culling_ratio"])))
    if cands.size > allowed:  # TopOpt.jl:449-460: stable sort by density
        cull = cands[np.argsort(new[cands], kind="stable")[:allowed]]
    else:
        cull = cands
    new[cull] = min_d
    if p.get("hard_update", 0):  # TopOpt.jl:464-472
        new[free & (new > min_d)] = f32(1.0)
    new[prot] = orig[prot]  # TopOpt.jl:474-479
    stats.update(active_count=active, candidates=int(cands.size), culled=int(cull.size))
    return new, stats

