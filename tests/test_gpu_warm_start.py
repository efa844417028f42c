"""Warm start across a refinement: the GPU displacement transfer
(hexa_remap_displacement) against the oracle, and a solve started from the
transferred field reaching the cold-start answer."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.refine import remap_displacement

pytestmark = pytest.mark.gpu


def test_displacement_transfer_matches_oracle_and_warm_starts(ctx, oracle, rng):
    from v119_2025_12_19_hexatop_aws_gb300 import workloads
    from v119_2025_12_19_hexatop_aws_gb300.solver import solve
    old, new = (16, 8, 8), (20, 10, 10)
    g0 = _lib.make_grid(*old, 1.0, 1.0, 1.0)
    g1 = _lib.make_grid(*new, 0.8, 0.8, 0.8)
    u = rng.standard_normal(3 * 17 * 9 * 9)
    out = remap_displacement(g0, g1, u, ctx=ctx)
    ref = oracle.remap_displacement(old, new, u)
    assert np.abs(out - ref).max() <= 1e-14 * np.abs(ref).max()
    # a warm start from the coarse solution reaches the same answer as a cold start
    p = _lib.default_params(precision="mixed", divergence_check=0, tol=1e-11)
    f0 = workloads.point_loads(*old, 1, seed=3)[0]
    u0, _ = solve(g0, np.ones(16 * 8 * 8), f0, clamp_faces=1, params=p, ctx=ctx)
    f1 = np.zeros(3 * 21 * 11 * 11)
    f1[3 * (20 + 21 * (5 + 11 * 0)) + 2] = -1.0
    cold, sc = solve(g1, np.ones(2000), f1, clamp_faces=1, params=p, ctx=ctx)
    warm, sw = solve(g1, np.ones(2000), f1, clamp_faces=1, params=p, ctx=ctx,
                     u_guess=remap_displacement(g0, g1, u0, ctx=ctx))
    assert sw["true_relres"] <= 1e-11 and sc["true_relres"] <= 1e-11
    assert np.linalg.norm(warm - cold) <= 1e-7 * np.linalg.norm(cold)

