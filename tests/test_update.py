"""The density update between solves (TopOpt.jl:211-482): the oracle's
restatement checked on hand-worked cases, without a GPU."""
import numpy as np
import pytest

F32 = np.float32


def params(**kw):
    p = dict(E=1.0, l1_stress_allowable=1.0, iter=1, number_of_iterations=30, min_density=1e-3, max_density=1.0,
             max_domain_dim=2.0, filter_R_init_perc=0.0, filter_R_interm_perc=0.0, filter_R_final_perc=0.0,
             filter_R_interm_iter_perc=50.0, minimum_filter_radius_as_elements=0.0, filter_tolerance=1e-5,
             final_density_threshold=0.95, max_culling_ratio=0.1, hard_update=0)
    p.update(kw)
    return p


def test_radius_schedule_follows_the_reference(oracle):
    # R from 10 % to 5 % of 2.0 over the first half (iterations 1..15), then to 2 %
    p = params(filter_R_init_perc=10.0, filter_R_interm_perc=5.0, filter_R_final_perc=2.0)
    r1, e1 = oracle.density_filter_radius(dict(p, iter=1), 0.01, 0.01, 0.01)
    assert r1 == F32(0.2) and e1 == F32(0.2) / F32(2.5)
    r15, _ = oracle.density_filter_radius(dict(p, iter=15), 0.01, 0.01, 0.01)
    assert r15 == F32(F32(5.0) / F32(100.0) * F32(2.0))
    r30, _ = oracle.density_filter_radius(dict(p, iter=30), 0.01, 0.01, 0.01)
    assert abs(float(r30) - 0.04) < 1e-7
    r99, _ = oracle.density_filter_radius(dict(p, iter=99), 0.01, 0.01, 0.01)
    assert r99 == r30  # iterations past the schedule keep the final radius
    # the floor at minimum_filter_radius_as_elements x mean element size
    rmin, _ = oracle.density_filter_radius(dict(p, iter=30, minimum_filter_radius_as_elements=2.5), 0.1, 0.1, 0.1)
    assert rmin == F32(2.5) * ((F32(0.1) + F32(0.1) + F32(0.1)) / F32(3.0))


def test_update_proposal_cull_and_projection(oracle):
    # 10 elements, none protected; proposal = l1 / allowable / E, floored at min_density
    l1 = np.array([0.0, 0.3, 0.5, 0.02, 0.9, 0.01, 0.6, 0.05, 2.0, 0.04], F32)
    dens = np.full(10, 0.5, F32)
    p = params(iter=30, max_culling_ratio=0.25, final_density_threshold=0.1)
    new, st = oracle.update_density(dens, l1, None, np.ones(10, F32), p, (0.1, 0.1, 0.1))
    # threshold 0.1 * 30/30; live: all but element 0 (0.001); candidates 0.02, 0.01, 0.05, 0.04
    assert st["current_threshold"] == F32(0.1) and st["active_count"] == 9 and st["candidates"] == 4
    # floor(9 * 0.25) = 2 culls: the two smallest, 0.01 (e5) and 0.02 (e3)
    assert st["culled"] == 2
    assert new[5] == F32(1e-3) and new[3] == F32(1e-3) and new[7] == F32(0.05) and new[9] == F32(0.04)
    assert new[8] == F32(1.0)  # clamped to max_density
    change = np.abs(np.minimum(np.maximum(l1, F32(1e-3)), F32(1.0)) - dens).astype(np.float64).sum()
    assert st["mean_change"] == F32(F32(change) / F32(9))
    hard, _ = oracle.update_density(dens, l1, None, np.ones(10, F32), dict(p, hard_update=1), (0.1, 0.1, 0.1))
    assert set(np.unique(hard)) == {F32(1e-3), F32(1.0)}


def test_update_ties_cull_lowest_index_first(oracle):
    l1 = np.array([0.05, 0.05, 0.5, 0.05, 0.05, 0.5, 0.5, 0.5], F32)
    p = params(iter=30, final_density_threshold=0.1, max_culling_ratio=0.3)
    new, st = oracle.update_density(np.full(8, 0.5, F32), l1, None, np.ones(8, F32), p, (0.1, 0.1, 0.1))
    assert st["candidates"] == 4 and st["culled"] == 2  # floor(8 * 0.3)
    assert list(np.nonzero(new == F32(1e-3))[0]) == [0, 1]


def test_update_protected_and_nan_paths(oracle):
    l1 = np.array([0.5, 0.5, 0.5, 0.5], F32)
    prot = np.array([1, 0, 0, 1], bool)
    orig = np.array([0.7, 1.0, 1.0, 0.0005], F32)
    new, st = oracle.update_density(np.full(4, 0.3, F32), l1, prot, orig, params(), (0.1, 0.1, 0.1))
    assert new[0] == F32(0.7) and new[3] == F32(0.0005) and new[1] == F32(0.5)
    assert st["active_count"] == 3  # protected counted by their original density
    bad = l1.copy()
    bad[2] = np.nan
    same, st = oracle.update_density(np.full(4, 0.3, F32), bad, prot, orig, params(), (0.1, 0.1, 0.1))
    assert st["status"] == 1 and np.all(same == F32(0.3))
    # a filter that returns NaN: the proposal is used instead
    p = params(filter_R_init_perc=10.0, filter_R_interm_perc=10.0, filter_R_final_perc=10.0)
    new2, st2 = oracle.update_density(np.full(4, 0.3, F32), l1, prot, orig, p, (0.1, 0.1, 0.1),
                                      filter_fn=lambda x, r: np.full_like(x, np.nan))
    assert st2["filter_used"] == 1 and st2["filter_nan_fallback"] == 1 and np.array_equal(new2, new)


def _update_loops(density, l1, prot, E, allow, it, n_it, orig, min_d, max_d, opt, h):
    """update_density! (TopOpt.jl:211-482) transcribed statement by statement
    in pure-Python loops over Float32 scalars, without a filter (R_effective
    at or below 1e-4): a cross-check of the vectorised restatement."""
    f32 = np.float32
    dens = [f32(v) for v in density]
    ne = len(dens)
    prop = [orig[e] if prot[e] else max((f32(l1[e]) / f32(allow)) / f32(E), f32(min_d)) for e in range(ne)]
    change, active1 = 0.0, 0
    for e in range(ne):
        if not prot[e]:
            old = dens[e]
            raw = max(prop[e], f32(min_d))
            dens[e] = raw
            change += float(abs(min(raw, f32(max_d)) - old))
            if dens[e] > f32(min_d):
                active1 += 1
    mean = f32(f32(change) / f32(active1)) if active1 > 0 else f32(0)
    if it > n_it:
        thr = f32(opt["final_density_threshold"])
    else:
        thr = f32(opt["final_density_threshold"]) * min(max(f32(it) / f32(n_it), f32(0)), f32(1))
    cands, active = [], 0
    for e in range(ne):
        if not prot[e]:
            if dens[e] > f32(max_d):
                dens[e] = f32(max_d)
            if dens[e] > f32(min_d):
                active += 1
                if dens[e] < thr:
                    cands.append(e)
        elif orig[e] > f32(min_d):
            active += 1
    allowed = int(np.floor(f32(active) * f32(opt["max_culling_ratio"])))
    if len(cands) > allowed:
        cands = sorted(cands, key=lambda e: dens[e])[:allowed]  # Python's sort is stable, as Julia's
    for e in cands:
        dens[e] = f32(min_d)
    if opt.get("hard_update"):
        for e in range(ne):
            if not prot[e] and dens[e] > f32(min_d):
                dens[e] = f32(1.0)
    for e in range(ne):
        if prot[e]:
            dens[e] = orig[e]
    return np.array(dens, np.float32), mean, active, len(cands)


@pytest.mark.parametrize("it,hard", [(3, 0), (30, 1), (45, 0)])
def test_vectorised_update_matches_the_loop_transcription(oracle, it, hard):
    rng = np.random.default_rng(it)
    ne = 600
    dens = rng.uniform(0, 1, ne).astype(F32)
    l1 = (rng.uniform(0, 1.5, ne) * 50).astype(F32)
    l1[rng.uniform(size=ne) < 0.3] = F32(0.5)  # ties
    prot = rng.uniform(size=ne) < 0.1
    orig = np.where(rng.uniform(size=ne) < 0.5, F32(1.0), F32(0.0)).astype(F32)
    p = params(E=50.0, iter=it, number_of_iterations=30, hard_update=hard, max_culling_ratio=0.2)
    new, st = oracle.update_density(dens, l1, prot, orig, p, (0.1, 0.1, 0.1))
    ref, mean, active, culled = _update_loops(dens, l1, prot, 50.0, 1.0, it, 30, orig, p["min_density"],
                                              p["max_density"], p, (0.1, 0.1, 0.1))
    assert np.array_equal(new, ref)
    assert st["active_count"] == active and st["culled"] == culled and st["mean_change"] == mean


def _radix_select_keys(keys, k, digit_bits=11):
    """The culling selection of csrc/update.cu in Python: six passes over
    the 64-bit keys (float bits << 32 | index), 11-bit digits from the top;
    each pass histograms the keys that share the prefix found so far and
    picks the digit holding the k-th smallest.  Returns the k-th smallest key."""
    prefix, remaining = 0, k
    top = 64
    while top > 0:
        width = digit_bits if top >= digit_bits else top
        shift = top - width
        above = shift + width
        hist = [0] * (1 << digit_bits)
        for key in keys:
            if above < 64 and (key >> above) != (prefix >> above):
                continue
            hist[(key >> shift) & ((1 << width) - 1)] += 1
        excl = 0
        for digit, cnt in enumerate(hist):
            if excl < remaining <= excl + cnt:
                prefix |= digit << shift
                remaining -= excl
                break
            excl += cnt
        top = shift
    return prefix


def test_radix_select_picks_the_stable_sort_prefix():
    rng = np.random.default_rng(3)
    for trial in range(40):
        n = int(rng.integers(1, 300))
        vals = rng.uniform(0.001, 0.9, n).astype(F32)
        if trial % 3 == 0:
            vals[rng.uniform(size=n) < 0.5] = F32(0.25)  # heavy ties
        if trial % 7 == 0:
            vals[:] = F32(0.5)  # all equal
        idx = np.sort(rng.choice(100000, n, replace=False))
        keys = [(int(np.float32(v).view(np.uint32)) << 32) | int(e) for v, e in zip(vals, idx)]
        order = sorted(range(n), key=lambda i: vals[i])  # stable: ties by index
        for k in {1, n, max(1, n // 3), max(1, n - 1)}:
            kth = _radix_select_keys(keys, k)
            chosen = {i for i in range(n) if keys[i] <= kth}
            assert chosen == set(order[:k]), (trial, n, k)


def test_dropin_reads_the_reference_config_keys(monkeypatch, built_lib):
    """topopt.update_density maps update_density!'s arguments and config keys
    (TopOpt.jl:238-300, 420-462) onto hexa_density_update_params; the GPU
    call is replaced by a recorder, so this runs anywhere."""
    from v119_2025_12_19_hexatop_aws_gb300 import topopt
    seen = {}

    def record(grid, density, l1, protected, original, params, ctx=None):
        seen.update(grid=(grid.nx, grid.ny, grid.nz, grid.dx), params=params)
        return dict(status=0, mean_change=0.5, R_length=0.25, current_threshold=0.125, filter_time=0.0,
                    filter_iters=3, filter_res=1e-6)

    monkeypatch.setattr(topopt, "update_density_gpu", record)
    config = {"optimization_parameters": {"filter_R_init_perc": 6.0, "filter_R_final_perc": 1.5,
                                          "max_culling_ratio": 0.05, "density_update_method": "hard",
                                          "final_density_threshold": 0.9},
              "solver_parameters": {"filter_tolerance": 1e-4},
              "geometry": {"nElem_x_computed": 8, "nElem_y_computed": 4, "nElem_z_computed": 2,
                           "dx_computed": 0.5, "dy_computed": 0.5, "dz_computed": 0.5, "max_domain_dim": 4.0}}
    out = topopt.update_density(np.zeros(64, F32), np.zeros(64, F32), None, F32(7.0), F32(2.0), 12, 40,
                                np.ones(64, F32), F32(0.01), F32(0.9), config)
    p = seen["params"]
    assert seen["grid"] == (8, 4, 2, 0.5)
    assert (p.E, p.l1_stress_allowable, p.iter, p.number_of_iterations) == (7.0, 2.0, 12, 40)
    assert p.min_density == F32(0.01) and p.max_density == F32(0.9) and p.max_domain_dim == 4.0
    assert p.filter_R_init_perc == 6.0 and p.filter_R_interm_perc == 0.0 and p.filter_R_final_perc == 1.5
    assert p.filter_R_interm_iter_perc == 50.0 and p.minimum_filter_radius_as_elements == 2.5
    assert p.filter_tolerance == F32(1e-4) and p.final_density_threshold == F32(0.9)
    assert p.max_culling_ratio == F32(0.05) and p.hard_update == 1
    assert out == (F32(0.5), F32(0.25), F32(0.125), 0.0, 3, 1e-6)
