"""hexa_filter_noalloc through the C ABI against hexa_filter.

The no-allocation entry point serves callers that cannot allocate device
memory where they filter (code running on its own stream while its
application captures another stream into a CUDA graph, or hosts whose own
pool owns the device-memory budget): its scratch lives in a fixed device array
inside the library.  Two calls in a row must give what the allocating entry
point gives, within this suite's filter tolerance; the grids run from the
larger to the smaller, so later calls start on leftovers of earlier, larger
calls beyond their own node count.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.helmholtz import filter_density

pytestmark = pytest.mark.gpu


def _noalloc(grid, rho_d, out_d, radius, tol, max_iter, quirk, stream=None):
    st = _lib.FilterStats()
    rc = _lib.load().hexa_filter_noalloc(C.byref(grid), rho_d.data_ptr(), float(radius), float(tol), int(max_iter),
                                         int(quirk), out_d.data_ptr(), stream, C.byref(st))
    return rc, st


def test_noalloc_filter_matches_allocating_filter_twice():
    torch = pytest.importorskip("torch")
    ctx = _lib.Context(0)
    try:
        # larger grid first: the second grid's calls run on what the first left in the array
        cases = [((48, 24, 24), 1.2, False, 8), ((24, 12, 12), 0.6, True, 7)]
        for dims, R, quirk, seed in cases:
            rng = np.random.default_rng(seed)
            grid = _lib.make_grid(*dims)
            ne = dims[0] * dims[1] * dims[2]
            for call in range(2):  # the second call reuses the array the first one left behind
                rho = rng.uniform(0.0, 1.0, ne)
                ref, ref_st = filter_density(grid, rho, R, tol=1e-10, max_iter=2000, quirk=quirk, ctx=ctx)
                rho_d = torch.from_numpy(rho).cuda()
                out_d = torch.full_like(rho_d, float("nan"))
                rc, st = _noalloc(grid, rho_d, out_d, R, 1e-10, 2000, quirk)
                assert rc == _lib.HEXA_OK, f"{dims} call {call}: status {rc}"
                out = out_d.cpu().numpy()
                assert np.abs(out - ref).max() <= 1e-10 * np.abs(ref).max(), f"{dims} call {call}"
                assert st.iterations == ref_st["iterations"]
    finally:
        ctx.close()


def test_noalloc_filter_allocates_nothing():
    """Device free memory is the same before and after a warmed-up call."""
    torch = pytest.importorskip("torch")
    dims = (32, 16, 16)
    grid = _lib.make_grid(*dims)
    rho_d = torch.from_numpy(np.random.default_rng(3).uniform(0, 1, 32 * 16 * 16)).cuda()
    out_d = torch.empty_like(rho_d)
    assert _noalloc(grid, rho_d, out_d, 0.8, 1e-9, 500, True)[0] == _lib.HEXA_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _noalloc(grid, rho_d, out_d, 0.8, 1e-9, 500, True)[0] == _lib.HEXA_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_filter_breakdown_gives_nan_like_hexa_filter():
    """A NaN in the input density: both entry points return a NaN field (the
    reference's callers test for it) after the same number of iterations."""
    torch = pytest.importorskip("torch")
    ctx = _lib.Context(0)
    try:
        dims = (12, 6, 6)
        grid = _lib.make_grid(*dims)
        rho = np.random.default_rng(5).uniform(0, 1, 12 * 6 * 6)
        rho[17] = np.nan
        ref, ref_st = filter_density(grid, rho, 0.6, tol=1e-8, max_iter=200, quirk=True, ctx=ctx)
        rho_d = torch.from_numpy(rho).cuda()
        out_d = torch.zeros_like(rho_d)
        rc, st = _noalloc(grid, rho_d, out_d, 0.6, 1e-8, 200, True)
        assert rc == _lib.HEXA_OK
        out = out_d.cpu().numpy()
        assert np.isnan(ref).all() and np.isnan(out).all()
        assert st.iterations == ref_st["iterations"]
    finally:
        ctx.close()


def test_noalloc_filter_runs_while_another_stream_captures():
    """The call runs on a non-blocking stream while this thread captures a
    graph on another stream (global capture mode): the capture stays valid, the
    graph replays, and the filtered field matches a call made outside any
    capture.  A capturing stream itself is refused."""
    torch = pytest.importorskip("torch")
    dims = (16, 8, 8)
    grid = _lib.make_grid(*dims)
    rho_d = torch.from_numpy(np.random.default_rng(9).uniform(0, 1, 16 * 8 * 8)).cuda()
    want_d = torch.empty_like(rho_d)
    out_d = torch.empty_like(rho_d)
    refused_d = torch.empty_like(rho_d)
    assert _noalloc(grid, rho_d, want_d, 0.7, 1e-10, 500, True)[0] == _lib.HEXA_OK  # outside any capture
    acc = torch.zeros(1024, device="cuda")
    side = torch.cuda.Stream()  # PyTorch creates its streams non-blocking
    graph = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    with torch.cuda.graph(graph, stream=cap):
        acc.add_(1.0)
        rc_side, _ = _noalloc(grid, rho_d, out_d, 0.7, 1e-10, 500, True, stream=side.cuda_stream)
        rc_cap, _ = _noalloc(grid, rho_d, refused_d, 0.7, 1e-10, 500, True, stream=cap.cuda_stream)
        still = torch.cuda.is_current_stream_capturing()
        acc.add_(1.0)
    assert rc_side == _lib.HEXA_OK
    assert rc_cap == _lib.HEXA_ERR_ARG
    assert still
    graph.replay()
    torch.cuda.synchronize()
    assert torch.all(acc == 2.0).item()
    assert torch.equal(out_d, want_d)


def test_noalloc_filter_rejects_oversized_grid_and_host_arrays():
    torch = pytest.importorskip("torch")
    big = _lib.make_grid(128, 64, 64)  # 545,025 nodes > HEXA_NOALLOC_MAX_NODES
    rho_d = torch.zeros(128 * 64 * 64, dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(big, rho_d, torch.empty_like(rho_d), 0.6, 1e-8, 100, True)
    assert rc == _lib.HEXA_ERR_TOO_LARGE
    small = _lib.make_grid(4, 4, 4)
    host = np.zeros(64)
    st = _lib.FilterStats()
    rc = _lib.load().hexa_filter_noalloc(C.byref(small), _lib.ptr(host), 0.6, 1e-8, 100, 1, _lib.ptr(host), None,
                                         C.byref(st))
    assert rc == _lib.HEXA_ERR_ARG
