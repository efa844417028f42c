"""The GPU field transfer onto a refined grid against the oracle's
restatement of MeshRefiner.jl:188-240 (Float32 both sides)."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.refine import domain_lengths, refine_mesh_and_fields, remap_fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("old,new,lengths", [((8, 4, 4), (13, 7, 6), (8.0, 4.0, 4.0)),
                                             ((20, 10, 10), (24, 12, 12), (2.0, 1.0, 1.0))])
def test_remap_matches_oracle(ctx, oracle, rng, old, new, lengths):
    n_old = old[0] * old[1] * old[2]
    dens = rng.uniform(0, 1, n_old).astype(np.float32)
    alpha = rng.uniform(-1, 1, n_old).astype(np.float32)
    h = tuple(L / n for L, n in zip(lengths, new))
    og = _lib.make_grid(*old, *(L / n for L, n in zip(lengths, old)))
    ng = _lib.make_grid(*new, *h)
    for projection in (False, True):
        nd, na = remap_fields(og, ng, lengths, dens, alpha, projection=projection, ctx=ctx)
        ref, ra, raw = oracle.remap_fields(old, new, (ng.dx, ng.dy, ng.dz), lengths, dens, alpha, projection)
        # every product and sum rounded once on both sides: bit-exact
        assert np.array_equal(nd, ref)
        assert np.array_equal(na, ra)


def test_refine_grows_the_grid(ctx, rng):
    grid = _lib.make_grid(16, 8, 8, 1.0, 1.0, 1.0)
    dens = np.where(rng.uniform(size=1024) < 0.5, 1.0, 0.001).astype(np.float32)
    g2, d2, a2, plan = refine_mesh_and_fields(grid, dens, None, 2000, domain_lengths(grid), max_growth_rate=1.5,
                                              memory_limit=10**7, ctx=ctx)
    assert plan.refine and g2.nx * g2.ny * g2.nz > 1024 and d2.size == g2.nx * g2.ny * g2.nz
    mid = (d2 >= np.float32(0.2)) & (d2 <= np.float32(0.4))
    assert np.all(mid | (d2 == np.float32(1e-4)) | (d2 == np.float32(1.0)))

