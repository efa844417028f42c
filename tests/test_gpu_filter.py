"""(d) The GPU Helmholtz filter against the oracle: the reference's own
Jacobi-PCG loop restated (GPUHelmholtz.jl:190-266) and the exact (LU) solve
of the same system (TopOpt.jl:32-127)."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.helmholtz import apply_gpu_filter, filter_density, radius_from_length

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(1, 1, 1), (6, 4, 3), (24, 12, 12), (33, 17, 9)])
@pytest.mark.parametrize("quirk", [True, False])
def test_filter_matches_exact(ctx, oracle, rng, dims, quirk):
    g = oracle.Grid(*dims)
    rho = rng.uniform(0, 1, g.nelem)
    R = 0.6
    ref = oracle.helmholtz_direct(g, rho, R, quirk=quirk)
    out, st = filter_density(_lib.make_grid(*dims), rho, R, tol=1e-14, max_iter=5000, quirk=quirk, ctx=ctx)
    assert np.abs(out - ref).max() <= 1e-10 * np.abs(ref).max()


def test_filter_follows_reference_loop(ctx, oracle, rng):
    dims = (24, 12, 12)
    g = oracle.Grid(*dims)
    rho = rng.uniform(0, 1, g.nelem)
    R = radius_from_length(2.5 * 1.5)
    ref, it_ref, res_ref = oracle.helmholtz_reference(g, rho, R, tol=1e-6, max_iter=200, quirk=True)
    out, st = filter_density(_lib.make_grid(*dims), rho, R, tol=1e-6, max_iter=200, quirk=True, ctx=ctx)
    assert st["iterations"] == it_ref
    assert st["relres"] == pytest.approx(res_ref, rel=1e-6)
    assert np.abs(out - ref).max() <= 1e-10


def test_filter_preserves_constants_on_true_brick(ctx, oracle):
    dims = (10, 6, 4)
    out, _ = filter_density(_lib.make_grid(*dims), np.full(240, 0.37), 1.2, tol=1e-14, max_iter=5000, quirk=False,
                            ctx=ctx)
    assert np.abs(out - 0.37).max() < 1e-12


def test_filter_quirk_scales_constants(ctx, oracle):
    # reference geometry: elements 1.5 dz tall with the nominal RHS volume -> constant / 1.5
    out, _ = filter_density(_lib.make_grid(8, 4, 4), np.full(128, 0.3), 0.7, tol=1e-14, max_iter=5000, quirk=True,
                            ctx=ctx)
    assert np.abs(out - 0.2).max() < 1e-12


def test_reference_signature_fp32(ctx, oracle, rng):
    dims = (12, 6, 6)
    g = oracle.Grid(*dims)
    rho = rng.uniform(0, 1, g.nelem).astype(np.float32)
    out, t, it, res = apply_gpu_filter(rho, *dims, 1.0, 1.0, 1.0, 0.6, None, 1e-6)
    ref, it_ref, _ = oracle.helmholtz_reference(g, rho.astype(np.float64), 0.6, tol=1e-6)
    assert out.dtype == np.float32 and out.shape == rho.shape
    assert abs(it - it_ref) <= 10
    assert np.abs(out - ref).max() < 1e-5


def test_zero_density_returns_input(ctx):
    out, st = filter_density(_lib.make_grid(4, 4, 4), np.zeros(64), 0.5, ctx=ctx)
    assert not out.any() and st["iterations"] == 0
