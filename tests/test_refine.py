"""Mesh growth: the refinement decision (host, MeshRefiner.jl:101-146,
Helpers.calculate_element_distribution) and the oracle's field transfer."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300.refine import element_distribution, plan_refinement


def test_element_distribution_keeps_cells_cubic():
    nx, ny, nz, dx, dy, dz, n = element_distribution(2.0, 1.0, 1.0, 16_000)
    assert (nx, ny, nz) == (40, 20, 20) and n == 16_000
    assert dx == dy == dz == np.float32(np.float32(2.0) / np.float32(40))
    # rounding per direction, at least one element each
    assert element_distribution(10.0, 1.0, 0.01, 1000)[:3] == (215, 22, 1)


def test_plan_follows_the_reference_limits():
    # already at the target: keep
    assert not plan_refinement(1000, 500, 400).refine
    # target-driven size 0.9 * 800 / 0.5 = 1440 vs growth limit 1200: growth wins
    p = plan_refinement(1000, 500, 800, max_growth_rate=1.2)
    assert p.refine and p.new_total == 1200 and p.limit == "Growth Rate Limit"
    # target-driven size below the growth limit
    p = plan_refinement(1000, 500, 600, max_growth_rate=2.0)
    assert p.refine and p.new_total == 1080 and p.limit == "Target Active Limit"
    # growth under 5 % is skipped
    assert not plan_refinement(1000, 500, 580, max_growth_rate=2.0).refine
    # memory and hard limits cap the size
    p = plan_refinement(1000, 100, 100_000, max_growth_rate=10.0, memory_limit=2000, hard_element_limit=5000)
    assert p.new_total == 2000 and p.limit == "RAM Limit"


def test_oracle_remap_preserves_constant_and_linear_fields(oracle):
    old = (8, 4, 4)
    const = np.full(128, 0.3, np.float32)
    val, _, raw = oracle.remap_fields(old, (16, 8, 8), (0.5, 0.5, 0.5), (8.0, 4.0, 4.0), const, projection=False)
    assert np.allclose(raw, 0.3, atol=1e-7)
    # a field linear in x is reproduced at interior centroids
    i = np.arange(128) % 8
    lin = (0.1 * i).astype(np.float32)
    val, _, raw = oracle.remap_fields(old, (16, 8, 8), (0.5, 0.5, 0.5), (8.0, 4.0, 4.0), lin, projection=False)
    ix = np.arange(16 * 64) % 16
    cx = (ix + 0.5) * 0.5  # new centroid; old cell-centre index space: cx - 0.5
    expect = 0.1 * np.clip(cx - 0.5, 0.0, 7.0)
    assert np.allclose(raw, expect, atol=1e-6)
    # projection thresholds
    pv, _, raw = oracle.remap_fields(old, (16, 8, 8), (0.5, 0.5, 0.5), (8.0, 4.0, 4.0), lin, projection=True)
    assert np.all(pv[raw > 0.4] == 1.0) and np.all(pv[raw < 0.2] == np.float32(1e-4))


def test_oracle_displacement_transfer_is_exact_on_trilinear_fields(oracle):
    old, new = (4, 2, 3), (7, 5, 4)

    def field(dims):
        nx, ny, nz = dims
        k, j, i = np.meshgrid(np.arange(nz + 1) / nz, np.arange(ny + 1) / ny, np.arange(nx + 1) / nx, indexing="ij")
        # trilinear in the box coordinates, one combination per component
        return np.stack([1 + 2 * i - j + 0.5 * i * j * k, 3 * k - i * k, j * k + 0.25], axis=-1).reshape(-1)
    out = oracle.remap_displacement(old, new, field(old))
    assert np.allclose(out, field(new), rtol=0, atol=1e-13)
    same = oracle.remap_displacement(old, old, field(old))
    assert np.array_equal(same, field(old))



def _remap_loops(old, new, new_h, lengths, density, alpha, projection):
    """MeshRefiner.jl:201-237 transcribed with its 1-based indices, one
    element at a time in Float32: a cross-check of the vectorised oracle."""
    f32 = np.float32
    onx, ony, onz = old
    nnx, nny, nnz = new
    nd, na = [], []
    for e_new in range(1, nnx * nny * nnz + 1):
        iz = (e_new - 1) // (nnx * nny) + 1
        rem = (e_new - 1) % (nnx * nny)
        iy = rem // nnx + 1
        ix = rem % nnx + 1
        cx = (f32(ix) - f32(0.5)) * f32(new_h[0])
        cy = (f32(iy) - f32(0.5)) * f32(new_h[1])
        cz = (f32(iz) - f32(0.5)) * f32(new_h[2])
        u = min(max((cx / f32(lengths[0])) * f32(onx), f32(0.5)), f32(onx) - f32(0.5))
        v = min(max((cy / f32(lengths[1])) * f32(ony), f32(0.5)), f32(ony) - f32(0.5))
        w = min(max((cz / f32(lengths[2])) * f32(onz), f32(0.5)), f32(onz) - f32(0.5))
        u0, v0, w0 = int(np.floor(u - f32(0.5))), int(np.floor(v - f32(0.5))), int(np.floor(w - f32(0.5)))
        tx, ty, tz = (u - f32(0.5)) - f32(u0), (v - f32(0.5)) - f32(v0), (w - f32(0.5)) - f32(w0)
        i0, i1 = min(max(u0 + 1, 1), onx), min(max(u0 + 2, 1), onx)
        j0, j1 = min(max(v0 + 1, 1), ony), min(max(v0 + 2, 1), ony)
        k0, k1 = min(max(w0 + 1, 1), onz), min(max(w0 + 2, 1), onz)

        def d(i, j, k):
            return f32(density[i + (j - 1) * onx + (k - 1) * onx * ony - 1])
        ctx, cty, ctz = (min(max(t, f32(0)), f32(1)) for t in (tx, ty, tz))
        one = f32(1)
        c00 = d(i0, j0, k0) * (one - ctx) + d(i1, j0, k0) * ctx
        c10 = d(i0, j1, k0) * (one - ctx) + d(i1, j1, k0) * ctx
        c01 = d(i0, j0, k1) * (one - ctx) + d(i1, j0, k1) * ctx
        c11 = d(i0, j1, k1) * (one - ctx) + d(i1, j1, k1) * ctx
        c0 = c00 * (one - cty) + c10 * cty
        c1 = c01 * (one - cty) + c11 * cty
        val = c0 * (one - ctz) + c1 * ctz
        if projection:
            val = f32(1.0) if val > f32(0.4) else (f32(0.0001) if val < f32(0.2) else val)
        nd.append(val)
        na.append(f32(alpha[i0 + (j0 - 1) * onx + (k0 - 1) * onx * ony - 1]))
    return np.array(nd, np.float32), np.array(na, np.float32)


@pytest.mark.parametrize("projection", [False, True])
def test_vectorised_remap_matches_the_loop_transcription(oracle, projection):
    rng = np.random.default_rng(5)
    old, new, L = (7, 4, 3), (9, 5, 4), (7.0, 4.0, 3.0)
    h = tuple(float(np.float32(np.float32(Li) / np.float32(n))) for Li, n in zip(L, new))
    dens = rng.uniform(0, 1, 84).astype(np.float32)
    alpha = rng.uniform(-1, 1, 84).astype(np.float32)
    nd, na, _ = oracle.remap_fields(old, new, h, L, dens, alpha, projection)
    rd, ra = _remap_loops(old, new, h, L, dens, alpha, projection)
    assert np.array_equal(nd, rd) and np.array_equal(na, ra)


def test_refine_entry_keeps_the_mesh_when_no_growth_is_due(monkeypatch):
    """refine_mesh_and_fields returns its inputs untouched when the reference
    would skip (target reached, growth under 5 %, memory limit after the
    distribution) and calls the transfer otherwise; the GPU call is recorded."""
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, refine
    calls = []

    def fake_remap(old, new, lengths, density, alpha=None, *, projection=True, ctx=None):
        calls.append((new.nx, new.ny, new.nz, projection))
        n = new.nx * new.ny * new.nz
        return np.zeros(n, np.float32), None if alpha is None else np.zeros(n, np.float32)

    monkeypatch.setattr(refine, "remap_fields", fake_remap)
    g = _lib.make_grid(10, 5, 5, 1.0, 1.0, 1.0)
    dens = np.full(250, 0.5, np.float32)
    L = refine.domain_lengths(g)
    out = refine.refine_mesh_and_fields(g, dens, None, 100, L)  # 250 active >= 100
    assert out[0] is g and out[1] is dens and not out[3].refine and not calls
    out = refine.refine_mesh_and_fields(g, dens, None, 1000, L, max_growth_rate=1.02)  # growth under 5 %
    assert out[0] is g and not calls
    out = refine.refine_mesh_and_fields(g, dens, None, 1000, L, max_growth_rate=2.0, memory_limit=260)
    assert out[0] is g and not calls  # the memory limit leaves growth under 5 %
    # 333 elements allowed, but the distribution rounds up to 11 x 6 x 6 = 396 (MeshRefiner.jl:151-155)
    assert refine.element_distribution(*L, 333)[6] == 396
    out = refine.refine_mesh_and_fields(g, dens, None, 1000, L, max_growth_rate=2.0, memory_limit=333)
    assert out[0] is g and not out[3].refine and not calls
    g2, d2, a2, plan = refine.refine_mesh_and_fields(g, dens, None, 1000, L, max_growth_rate=2.0,
                                                     update_method="soft")
    assert plan.refine and calls == [(g2.nx, g2.ny, g2.nz, False)] and d2.size == g2.nx * g2.ny * g2.nz
