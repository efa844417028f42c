"""(f) Stress post-processing on the GPU against the oracle's restatement of
Stress.stress_kernel! (Stress.jl:159-285): Float32 on both sides, so the bar
is a few Float32 roundings of each element's own stress scale."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads
from v119_2025_12_19_hexatop_aws_gb300.solver import solve
from v119_2025_12_19_hexatop_aws_gb300.topopt import stress_field

pytestmark = pytest.mark.gpu


def compare(out, ref, scale):
    tol = 1e-4 * scale + 1e-30
    assert np.all(np.abs(out["principal"] - ref["principal"]) <= tol[:, None])
    assert np.all(np.abs(out["voigt"] - ref["voigt"]) <= tol[:, None])
    assert np.all(np.abs(out["vonmises"] - ref["vonmises"]) <= 2 * tol)
    assert np.all(np.abs(out["l1"] - ref["l1"]) <= 3 * tol)
    # directions: where the extreme eigenvalues are well separated from the middle one
    p = ref["principal"]
    for key, gap in (("dir_max", p[:, 0] - p[:, 1]), ("dir_min", p[:, 1] - p[:, 2])):
        sep = gap > 1e-2 * scale
        dots = np.abs(np.sum(out[key][sep] * ref[key][sep], axis=1))
        assert np.all(dots >= 0.999), key


@pytest.mark.parametrize("dims,h", [((6, 4, 3), (1.0, 1.0, 1.0)), ((20, 10, 8), (1.0, 2.0, 0.5))])
def test_stress_matches_oracle_random_fields(ctx, oracle, rng, dims, h):
    g = oracle.Grid(*dims, *h)
    u = 1e-2 * rng.standard_normal(g.ndof)
    dens = rng.uniform(0.0, 1.0, g.nelem).astype(np.float32)
    dens[::7] = 1e-7  # below the reference's 1e-6 cut: zero output
    out = stress_field(_lib.make_grid(*dims, *h), u, dens, E=2.5, nu=0.3, ctx=ctx)
    ref = oracle.stress_field(g, u, dens, 2.5, 0.3)
    scale = np.abs(ref["voigt"]).max(axis=1)
    compare(out, ref, scale)
    assert not out["principal"][::7].any() and not out["vonmises"][::7].any()
    assert np.all(out["principal"][:, 0] >= out["principal"][:, 1])
    assert np.all(out["principal"][:, 1] >= out["principal"][:, 2])


def test_stress_of_a_solved_cantilever(ctx, oracle):
    dims = (24, 12, 12)
    g = oracle.Grid(*dims)
    rho = np.clip(workloads.c1_density(*dims), 0.0, 1.0)
    fac = 1e-9 + rho ** 3 * (1 - 1e-9)
    f = workloads.edge_load(*dims)
    u, st = solve(_lib.make_grid(*dims), fac, f, clamp_faces=1, params=_lib.default_params(divergence_check=0), ctx=ctx)
    assert st["status"] == 0
    dens = rho.astype(np.float32)
    out = stress_field(_lib.make_grid(*dims), u, dens, E=1.0, nu=0.3, ctx=ctx)
    ref = oracle.stress_field(g, u, dens, 1.0, 0.3)
    compare(out, ref, np.abs(ref["voigt"]).max(axis=1))
    # the principal stresses are the eigenvalues of the Voigt stress tensor
    v = ref["voigt"].astype(np.float64)
    S = np.zeros((g.nelem, 3, 3))
    S[:, 0, 0], S[:, 1, 1], S[:, 2, 2] = v[:, 0], v[:, 1], v[:, 2]
    S[:, 0, 1] = S[:, 1, 0] = v[:, 3]
    S[:, 1, 2] = S[:, 2, 1] = v[:, 4]
    S[:, 0, 2] = S[:, 2, 0] = v[:, 5]
    w = np.sort(np.linalg.eigvalsh(S), axis=1)[:, ::-1]
    assert np.abs(out["principal"] - w).max() <= 1e-4 * np.abs(w).max()


def test_reference_signature_mirror(ctx, rng):
    from v119_2025_12_19_hexatop_aws_gb300.mesh import generate_mesh
    from v119_2025_12_19_hexatop_aws_gb300.topopt import compute_stress_field
    dims = (6, 4, 3)
    nodes, elements, _ = generate_mesh(*dims, 1.0, 1.0, 1.0)
    ne, nn = 72, 7 * 5 * 4
    U = (1e-2 * rng.standard_normal(3 * nn)).astype(np.float32)
    dens = rng.uniform(0.0, 1.0, ne).astype(np.float32)
    pr, vm, vo, l1, dmax, dmin = compute_stress_field(nodes, elements, U, np.float32(2.0), np.float32(0.3), dens, ctx=ctx)
    ref = stress_field(_lib.make_grid(*dims), U.astype(np.float64), dens, E=2.0, nu=0.3, ctx=ctx)
    assert pr.shape == (3, ne) and vo.shape == (6, ne) and dmax.shape == (3, ne)
    assert np.array_equal(pr, ref["principal"].T) and np.array_equal(vm, ref["vonmises"])
    assert np.array_equal(l1, ref["l1"]) and np.array_equal(dmin, ref["dir_min"].T)
    _, _, none, _, _, _ = compute_stress_field(nodes, elements, U, 2.0, 0.3, dens, return_voigt=False, ctx=ctx)
    assert none.shape == (0, 0)
