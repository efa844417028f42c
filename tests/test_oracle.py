"""The oracle itself, on CPU: first-principles checks of the restated
reference operators and solvers (the reference ships no tests to pin them)."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import workloads


def test_operator_symmetric_and_matches_assembly(oracle, rng):
    g = oracle.Grid(5, 3, 4)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    fac = rng.uniform(0.1, 1, g.nelem)
    x, y = rng.standard_normal(g.ndof), rng.standard_normal(g.ndof)
    Kx, Ky = oracle.apply_K(g, K0, fac, x), oracle.apply_K(g, K0, fac, y)
    assert abs(y @ Kx - x @ Ky) < 1e-12 * abs(y @ Kx)
    K = oracle.assemble_K(g, K0, fac)
    assert np.abs(K @ x - Kx).max() < 1e-13 * np.abs(Kx).max()


def test_rigid_translation_null(oracle, rng):
    g = oracle.Grid(4, 4, 3)
    K0 = oracle.canonical_stiffness(1, 2, 1, 0.3)
    y = oracle.apply_K(g, K0, rng.uniform(0.1, 1, g.nelem), np.tile([0.0, 1.0, 0.0], g.nnode))
    assert np.abs(y).max() < 1e-13


def test_patch_uniform_strain_interior_residual_zero(oracle):
    g = oracle.Grid(6, 5, 4)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    NX, NY, NZ = 7, 6, 5
    k, j, i = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    u = np.stack([0.01 * i.ravel() + 0.002 * j.ravel(), -0.003 * k.ravel(), 0.004 * i.ravel()], 1).ravel()
    y = oracle.apply_K(g, K0, np.ones(g.nelem), u).reshape(NZ, NY, NX, 3)
    assert np.abs(y[1:-1, 1:-1, 1:-1]).max() < 1e-15


def test_reference_pcg_matches_direct(oracle, rng):
    g = oracle.Grid(8, 4, 4)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    fac = rng.uniform(0.2, 1, g.nelem)
    fixed = oracle.fixed_mask(g, 1)
    f = workloads.edge_load(8, 4, 4)
    # at 1e-9 the reference's absolute |p.Ap| < 1e-20 breakdown test (GPUSolver.jl:374) is not reached
    u, rel, info = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-9, max_iter=10000, shift_factor=1e-10)
    sigma = info.shifts[0]
    ud = oracle.direct_solve(g, K0, fac, f, fixed, sigma)
    assert info.success and rel < 1e-9 and len(info.shifts) == 1
    assert np.linalg.norm(u - ud) < 1e-7 * np.linalg.norm(ud)
    # tighter, the breakdown test stops every attempt: the reference's own behaviour
    _, rel2, info2 = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-14, max_iter=10000, shift_factor=1e-10)
    assert not info2.success and len(info2.shifts) == 3
    ut, relt, _ = oracle.cg_tight(g, K0, fac, f, fixed, sigma)
    assert np.linalg.norm(ut - ud) < 1e-10 * np.linalg.norm(ud)


def test_reference_pcg_failure_paths(oracle, rng):
    g = oracle.Grid(8, 4, 4)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    fac = rng.uniform(0.2, 1, g.nelem)
    fixed = oracle.fixed_mask(g, 1)
    f = workloads.edge_load(8, 4, 4)
    u, rel, info = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-12, max_iter=3, shift_factor=1e-10,
                                        max_shift_attempts=2, shift_multiplier=4.0)
    assert not info.success and len(info.shifts) == 2 and info.shifts[1] == pytest.approx(4 * info.shifts[0])
    u2, rel2, info2 = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-12, max_iter=10, shift_factor=1e-10,
                                           stagnation_tol=100.0)
    assert info2.success
    bad = fac.copy()
    bad[3] = np.nan
    _, r3, i3 = oracle.pcg_reference(g, K0, bad, f, fixed, tol=1e-9, max_iter=10, shift_factor=1e-10)
    assert i3.name == "Failed_Corrupt_Input" and np.isnan(r3)


def test_reference_multigrid_preconditioner(oracle, rng):
    """The restated two-level preconditioner of GPUGeometricMultigrid.jl."""
    g = oracle.Grid(8, 4, 4)
    fixed = oracle.fixed_mask(g, 1)
    free = ~fixed
    mg = oracle.ReferenceMG(g, free)
    assert mg.nc == (4, 2, 2)
    # even grids: every fine node's trilinear weights sum to 1 (nothing falls outside)
    wsum = np.zeros(g.nnode, np.float32)
    for nodes, _, w in mg.corners:
        np.add.at(wsum, nodes, w)
    assert np.allclose(wsum, 1.0, atol=1e-7)
    # D_c = 1 + (adjacent coarse elements) x the x-diagonal of the unit coarse K0
    kd = np.diag(oracle.canonical_stiffness(2, 2, 2, 0.3, fp32=True))[0]
    assert mg.Dc[0] == np.float32(1.0) + np.float32(kd)  # a corner node: one element
    # symmetric positive (additive Jacobi + P D_c^-1 P^T), to Float32 rounding
    n = int(free.sum())
    Minv = rng.uniform(0.5, 1.0, n)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    Ma, Mb = mg.apply(a, Minv), mg.apply(b, Minv)
    assert abs(b @ Ma - a @ Mb) <= 1e-5 * abs(b @ Ma) and a @ Ma > 0
    # odd grids drop the weight of coarse nodes beyond the coarse grid, as the reference's range test does
    g3 = oracle.Grid(5, 3, 3)
    mg3 = oracle.ReferenceMG(g3, ~oracle.fixed_mask(g3, 1))
    w3 = np.zeros(g3.nnode, np.float32)
    for nodes, _, w in mg3.corners:
        np.add.at(w3, nodes, w)
    assert w3.min() < 1.0 and w3.max() == np.float32(1.0)


def test_reference_multigrid_pcg_matches_direct(oracle, rng):
    g = oracle.Grid(8, 4, 4)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    fac = rng.uniform(0.2, 1, g.nelem)
    fixed = oracle.fixed_mask(g, 1)
    f = workloads.edge_load(8, 4, 4)
    # the preconditioned residual of this unit load meets the reference's absolute
    # |p.Ap| < 1e-20 breakdown test near relres 2e-8 (GPUSolver.jl:374), so 1e-7 here
    u, rel, info = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-7, max_iter=10000, shift_factor=1e-10,
                                        precond="multigrid")
    assert info.success and info.name == "GMG_GPU" and rel < 1e-7
    ud = oracle.direct_solve(g, K0, fac, f, fixed, info.shifts[0])
    assert np.linalg.norm(u - ud) < 1e-5 * np.linalg.norm(ud)
    _, rel9, i9 = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-9, max_iter=10000, shift_factor=1e-10,
                                       precond="multigrid")
    assert not i9.success and len(i9.shifts) == 3 and rel9 < 1e-7  # every attempt ends in that test
    _, _, ij = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-9, max_iter=10000, shift_factor=1e-10)
    assert ij.name == "Jacobi_GPU"


def test_reference_multigrid_falls_back_to_jacobi(oracle, rng, monkeypatch):
    """A NaN from the multigrid preconditioner restarts every attempt with
    Jacobi (GPUSolver.jl:389-437); the fault is planted in the oracle's MG."""
    g = oracle.Grid(8, 4, 4)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    fac = rng.uniform(0.2, 1, g.nelem)
    fixed = oracle.fixed_mask(g, 1)
    f = workloads.edge_load(8, 4, 4)
    monkeypatch.setattr(oracle.ReferenceMG, "apply", lambda self, r, Minv: np.full_like(r, np.nan))
    u, rel, info = oracle.pcg_reference(g, K0, fac, f, fixed, tol=1e-9, max_iter=10000, shift_factor=1e-10,
                                        precond="multigrid")
    assert info.success and info.name == "Jacobi_GPU" and rel < 1e-9
    assert len(info.iterations) == 2 and info.iterations[0] == 1  # MG stopped at the first check


def test_helmholtz_reference_vs_direct(oracle, rng):
    g = oracle.Grid(10, 6, 4)
    rho = rng.uniform(0, 1, g.nelem)
    ref, it, rel = oracle.helmholtz_reference(g, rho, 0.6, tol=1e-12, max_iter=500)
    d = oracle.helmholtz_direct(g, rho, 0.6)
    assert np.abs(ref - d).max() < 1e-10 and it % 10 == 0


@pytest.mark.parametrize("quirk", [True, False])
def test_helmholtz_c_loop_matches_numpy_loop(oracle, rng, quirk):
    """The C restatement of the filter's Jacobi-PCG (used where the numpy loop
    is too slow, e.g. to make the 384x192x192 densities on the host) takes the
    same iterations and gives the same field as the numpy loop."""
    g = oracle.Grid(13, 7, 5)
    rho = rng.uniform(0, 1, g.nelem)
    ref, it_ref, rel_ref = oracle.helmholtz_reference(g, rho, 1.1, 1e-10, max_iter=500, quirk=quirk)
    out, it, rel = oracle.helmholtz_pcg_c(g, rho, 1.1, 1e-10, max_iter=500, quirk=quirk)
    assert it == it_ref
    assert rel == pytest.approx(rel_ref, rel=1e-6)
    assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()
    z, itz, _ = oracle.helmholtz_pcg_c(g, np.zeros(g.nelem), 1.1, 1e-10)
    assert itz == 0 and not z.any()


def test_oc_volume_and_bounds(oracle, rng):
    x = rng.uniform(0, 1, 1000)
    dc = -rng.uniform(0.1, 2, 1000)
    xn, lam = oracle.oc_update(x, dc, np.ones(1000), 0.4, move=0.2)
    assert abs(xn.mean() - 0.4) < 1e-9 and lam > 0
    assert np.all(xn >= np.maximum(0, x - 0.2) - 1e-15) and np.all(xn <= np.minimum(1, x + 0.2) + 1e-15)


def test_cpu_baseline_converges_float32(oracle, rng):
    g = oracle.Grid(8, 4, 4)
    dens = rng.uniform(0.2, 1, g.nelem).astype(np.float32)
    f = workloads.edge_load(8, 4, 4).astype(np.float32)
    fixed = oracle.fixed_mask(g, 1).astype(np.uint8)
    u, rel, it, sec = oracle.cpu_matrix_free_cg(g, 1.0, dens, f, fixed, max_iter=5000, tol=1e-5, shift_factor=1e-10,
                                                nthreads=2)
    assert rel < 1e-5 and it > 10
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    fx = oracle.fixed_mask(g, 1)
    ud = oracle.direct_solve(g, K0, dens.astype(np.float64), f.astype(np.float64), fx,
                             1e-10 * oracle.diag_K(g, K0, dens.astype(np.float64), quirk=False)[~fx].max())
    assert np.linalg.norm(u - ud) < 1e-3 * np.linalg.norm(ud)
    assert np.all(u[fx] == 0)


def test_cpu_baseline_skips_soft_elements(oracle):
    # CPUSolver.jl:82: elements with density < min_stiffness_threshold are left out
    g = oracle.Grid(4, 2, 2)
    dens = np.full(g.nelem, 0.5, dtype=np.float32)
    dens[:4] = 1e-6
    f = workloads.edge_load(4, 2, 2).astype(np.float32)
    fixed = oracle.fixed_mask(g, 1).astype(np.uint8)
    u1, *_ = oracle.cpu_matrix_free_cg(g, 1.0, dens, f, fixed, max_iter=5, tol=1e-30, nthreads=1)
    dens2 = dens.copy()
    dens2[:4] = 0.0
    u2, *_ = oracle.cpu_matrix_free_cg(g, 1.0, dens2, f, fixed, max_iter=5, tol=1e-30, nthreads=1)
    assert np.array_equal(u1, u2)


def test_stress_oracle_principal_stresses_are_eigenvalues(oracle, rng):
    g = oracle.Grid(5, 4, 3, 1.0, 2.0, 0.5)
    u = 1e-2 * rng.standard_normal(g.ndof)
    dens = rng.uniform(0.0, 1.0, g.nelem).astype(np.float32)
    out = oracle.stress_field(g, u, dens, 1.0, 0.3)
    v = out["voigt"].astype(np.float64)
    S = np.zeros((g.nelem, 3, 3))
    S[:, 0, 0], S[:, 1, 1], S[:, 2, 2] = v[:, 0], v[:, 1], v[:, 2]
    S[:, 0, 1] = S[:, 1, 0] = v[:, 3]
    S[:, 1, 2] = S[:, 2, 1] = v[:, 4]
    S[:, 0, 2] = S[:, 2, 0] = v[:, 5]
    w, vec = np.linalg.eigh(S)
    assert np.abs(out["principal"] - w[:, ::-1]).max() <= 1e-5 * np.abs(w).max()
    # the directions are unit eigenvectors of the largest and smallest
    for key, col in (("dir_max", 2), ("dir_min", 0)):
        d = out[key].astype(np.float64)
        assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
        assert np.all(np.abs(np.sum(d * vec[:, :, col], axis=1)) >= 1 - 1e-4)


def _eigen3x3_loops(s11, s22, s33, s12, s23, s13):
    """eigen3x3_device (Stress.jl:95-157) transcribed statement by statement
    on Float32 scalars: a cross-check of the vectorised restatement."""
    f = np.float32
    s11, s22, s33, s12, s23, s13 = (f(x) for x in (s11, s22, s33, s12, s23, s13))
    v = [[f(1), f(0), f(0)], [f(0), f(1), f(0)], [f(0), f(0), f(1)]]

    def rot(spp, sqq, spq, spr, sqr, p, q):
        h = spq
        g = f(100) * abs(h)
        if abs(spp) + g != abs(spp) or abs(sqq) + g != abs(sqq):
            theta = f(0.5) * (sqq - spp) / h
            t = f(1) / (abs(theta) + np.sqrt(theta * theta + f(1)))
            if theta < f(0):
                t = -t
            c = f(1) / np.sqrt(t * t + f(1))
            s = t * c
            tau = s / (f(1) + c)
            spp, sqq = spp - t * spq, sqq + t * spq
            spq = f(0)
            tmp = spr
            spr = spr - s * (sqr + tau * spr)
            sqr = sqr + s * (tmp - tau * sqr)
            for r in range(3):
                vp = v[r][p]
                v[r][p] = vp - s * (v[r][q] + tau * vp)
                v[r][q] = v[r][q] + s * (vp - tau * v[r][q])
        return spp, sqq, spq, spr, sqr

    with np.errstate(over="ignore"):
        for _ in range(12):
            if max(abs(s12), abs(s23), abs(s13)) < f(1e-9):
                break
            s11, s22, s12, s13, s23 = rot(s11, s22, s12, s13, s23, 0, 1)
            s11, s33, s13, s12, s23 = rot(s11, s33, s13, s12, s23, 0, 2)
            s22, s33, s23, s12, s13 = rot(s22, s33, s23, s12, s13, 1, 2)
    ev = [s11, s22, s33]
    for a, b in ((0, 1), (1, 2), (0, 1)):
        if ev[a] < ev[b]:
            ev[a], ev[b] = ev[b], ev[a]
            for r in range(3):
                v[r][a], v[r][b] = v[r][b], v[r][a]
    return np.array(ev, np.float32), np.array([v[r][0] for r in range(3)]), np.array([v[r][2] for r in range(3)])


def test_vectorised_eigen_matches_the_loop_transcription(oracle):
    rng = np.random.default_rng(21)
    n = 300
    t = (rng.standard_normal((6, n)) * np.float32(1e3)).astype(np.float32)
    t[3:, :20] = 0.0  # already diagonal
    t[:, 20:40] = t[:, 20:21]  # repeated tensors
    t[4, 40:60] = np.float32(1e-12)  # nearly diagonal
    vals, vmax, vmin = oracle.eigen3x3(*t)
    for e in range(n):
        ev, dmax, dmin = _eigen3x3_loops(*t[:, e])
        assert np.array_equal(vals[e], ev), e
        assert np.array_equal(vmax[e], dmax) and np.array_equal(vmin[e], dmin), e
