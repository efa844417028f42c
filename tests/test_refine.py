"""Mesh growth: the refinement decision (host, MeshRefiner.jl:101-146,
Helpers.calculate_element_distribution) and the oracle's field transfer."""
import numpy as np

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

