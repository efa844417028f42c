"""hexa_filter_noalloc through the C ABI against hexa_filter.

The no-allocation entry point serves callers that cannot allocate device
memory where they filter (code running while its application captures a CUDA
stream, or hosts whose own pool owns the device-memory budget): its scratch
lives in a fixed device array inside the library.  Two calls in a row must
give what the allocating entry point gives, within this suite's filter
tolerance, the second call starting from the first call's leftovers in the
shared array.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.helmholtz import filter_density

pytestmark = pytest.mark.gpu


def _noalloc(grid, rho_d, out_d, radius, tol, max_iter, quirk):
    st = _lib.FilterStats()
    rc = _lib.load().hexa_filter_noalloc(C.byref(grid), rho_d.data_ptr(), float(radius), float(tol), int(max_iter),
                                         int(quirk), out_d.data_ptr(), None, C.byref(st))
    return rc, st


def test_noalloc_filter_matches_allocating_filter_twice():
    torch = pytest.importorskip("torch")
    ctx = _lib.Context(0)
    try:
        cases = [((24, 12, 12), 0.6, True, 7), ((40, 20, 16), 1.2, False, 8)]
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
                assert rc == _lib.HEXA_OK, f"call {call}: status {rc}"
                out = out_d.cpu().numpy()
                assert np.abs(out - ref).max() <= 1e-10 * np.abs(ref).max(), f"call {call}"
                assert st.iterations == ref_st["iterations"]
    finally:
        ctx.close()


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
