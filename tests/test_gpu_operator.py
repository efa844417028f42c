"""(a) The node-centric GPU operator against the oracle's element scatter
(GPUSolver.jl:91-128 restated), through the C ABI."""
import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.solver import apply_operator, operator_diagonal

pytestmark = pytest.mark.gpu

# (62, 15, 20) and (64, 32, 12) have tiles whose columns all lie inside the
# grid (the predicate-free item path of the kernel), besides boundary tiles
GRIDS = [(1, 1, 1), (2, 1, 1), (4, 2, 2), (5, 3, 7), (33, 17, 9), (62, 15, 20), (31, 7, 3), (64, 32, 12)]


def _case(oracle, rng, dims, h=(1.0, 1.0, 1.0), faces=1, nodemask=False):
    g = oracle.Grid(*dims, *h)
    fac = rng.uniform(1e-3, 1.0, g.nelem)
    x = rng.standard_normal(g.ndof)
    fixed_dof = None
    if nodemask:
        fixed_dof = (rng.uniform(size=g.ndof) < 0.05).astype(np.uint8)
    fixed = oracle.fixed_mask(g, faces, fixed_dof)
    return g, fac, x, fixed_dof, fixed


@pytest.mark.parametrize("dims", GRIDS)
@pytest.mark.parametrize("sigma", [0.0, 1e-3])
def test_apply_fp64_matches_oracle(ctx, oracle, rng, dims, sigma):
    g, fac, x, fd, fixed = _case(oracle, rng, dims, faces=1)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    y_ref = oracle.apply_A(g, K0, fac, x, fixed, sigma)
    y = apply_operator(_lib.make_grid(*dims), fac, x, nu=0.3, sigma=sigma, clamp_faces=1, ctx=ctx)
    scale = np.abs(y_ref).max()
    assert np.abs(y - y_ref).max() <= 1e-13 * scale


@pytest.mark.parametrize("dims", [(5, 3, 7), (33, 17, 9), (64, 32, 6)])
def test_apply_brick_nodemask_faces(ctx, oracle, rng, dims):
    h = (1.0, 2.0, 0.5)
    g, fac, x, fd, fixed = _case(oracle, rng, dims, h=h, faces=0b010110, nodemask=True)
    K0 = oracle.canonical_stiffness(*h, 0.25)
    y_ref = oracle.apply_A(g, K0, fac, x, fixed, 0.0)
    y = apply_operator(_lib.make_grid(*dims, *h), fac, x, nu=0.25, clamp_faces=0b010110, fixed_dof=fd, ctx=ctx)
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()


@pytest.mark.parametrize("dims", [(4, 2, 2), (33, 17, 9), (64, 32, 12)])
def test_apply_fp32_matches_oracle(ctx, oracle, rng, dims):
    g, fac, x, fd, fixed = _case(oracle, rng, dims, faces=1)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    y_ref = oracle.apply_A(g, K0, fac.astype(np.float32).astype(np.float64), x.astype(np.float32).astype(np.float64), fixed)
    y = apply_operator(_lib.make_grid(*dims), fac.astype(np.float32), x.astype(np.float32), clamp_faces=1, ctx=ctx,
                       fp32=True)
    assert np.abs(y.astype(np.float64) - y_ref).max() <= 2e-6 * np.abs(y_ref).max()


def test_apply_is_deterministic(ctx, oracle, rng):
    g, fac, x, fd, fixed = _case(oracle, rng, (40, 20, 20))
    grid = _lib.make_grid(40, 20, 20)
    y1 = apply_operator(grid, fac, x, clamp_faces=1, ctx=ctx)
    y2 = apply_operator(grid, fac, x, clamp_faces=1, ctx=ctx)
    assert np.array_equal(y1, y2)


def test_rigid_body_modes_are_in_the_kernel(ctx, oracle, rng):
    dims = (9, 5, 6)
    g = oracle.Grid(*dims)
    fac = rng.uniform(0.1, 1.0, g.nelem)
    NX, NY, NZ = dims[0] + 1, dims[1] + 1, dims[2] + 1
    k, j, i = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    X = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(np.float64)
    modes = [np.tile([1.0, 0, 0], g.nnode), np.stack([-X[:, 1], X[:, 0], 0 * X[:, 0]], 1).ravel()]
    for u in modes:
        y = apply_operator(_lib.make_grid(*dims), fac, u, ctx=ctx)
        assert np.abs(y).max() < 1e-12 * np.abs(u).max()


def test_ignores_values_at_fixed_dofs(ctx, oracle, rng):
    g, fac, x, fd, fixed = _case(oracle, rng, (6, 4, 4))
    x2 = x.copy()
    x2[fixed] = 1e6
    grid = _lib.make_grid(6, 4, 4)
    assert np.array_equal(apply_operator(grid, fac, x, clamp_faces=1, ctx=ctx),
                          apply_operator(grid, fac, x2, clamp_faces=1, ctx=ctx))


@pytest.mark.parametrize("quirk", [0, 1])
def test_diagonal_matches_oracle(ctx, oracle, rng, quirk):
    dims, h = (7, 5, 3), (1.0, 2.0, 0.5)
    g = oracle.Grid(*dims, *h)
    fac = rng.uniform(0.01, 1, g.nelem)
    K0 = oracle.canonical_stiffness(*h, 0.3)
    d_ref = oracle.diag_K(g, K0, fac, quirk=bool(quirk))
    d_ref[oracle.fixed_mask(g, 1)] = 0
    d = operator_diagonal(_lib.make_grid(*dims, *h), fac, clamp_faces=1, diag_quirk=quirk, ctx=ctx)
    assert np.abs(d - d_ref).max() <= 1e-14 * d_ref.max()


@pytest.mark.parametrize("dims", [(5, 3, 7), (33, 17, 9)])
def test_timed_chebyshev_step_reads_its_previous_iterate(ctx, oracle, rng, dims):
    """hexa_time_operator's mode 5 is the smoother's Chebyshev step written in
    place over its previous iterate y (one warm-up launch, then `reps`), so the
    benchmark's roofline times the kernel the V-cycle runs, x_prev stream
    included: y <- x + 0.5 (x - y) + 0.3 D^-1 (b - A x), D the x-diagonal form."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    g, fac, x, fd, fixed = _case(oracle, rng, dims)
    x[fixed] = 0.0
    b = rng.standard_normal(g.ndof)
    b[fixed] = 0.0
    y0 = rng.standard_normal(g.ndof)
    f32 = lambda a: a.astype(np.float32)
    fac, x, b, y0 = f32(fac), f32(x), f32(b), f32(y0)
    K0 = oracle.canonical_stiffness(1, 1, 1, 0.3)
    ax = oracle.apply_A(g, K0, fac.astype(np.float64), x.astype(np.float64), fixed)
    d = oracle.diag_K(g, K0, fac.astype(np.float64), quirk=True)
    dinv = np.where(fixed, 0.0, 1.0 / np.where(fixed, 1.0, d))
    reps = 2
    want = y0.astype(np.float64)
    for _ in range(reps + 1):
        want = np.where(fixed, 0.0, x + 0.5 * (x - want) + 0.3 * dinv * (b - ax))
    dev = lambda a: torch.from_numpy(a).cuda()
    fac_d, x_d, b_d, y_d = dev(fac), dev(x), dev(b), dev(y0.copy())
    t = C.c_double()
    bc = _lib.make_bc(1)
    rc = ctx.lib.hexa_time_operator(ctx.h, C.byref(_lib.make_grid(*dims)), C.byref(bc), 0.3, 2, 5, fac_d.data_ptr(),
                                    x_d.data_ptr(), b_d.data_ptr(), y_d.data_ptr(), reps, C.byref(t))
    assert rc == _lib.HEXA_OK and t.value > 0
    got = y_d.cpu().numpy().astype(np.float64)
    assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max()


def test_staged_operator_wait_that_runs_out_is_reported():
    """Every wait of the TMA-staged FP32 operator (HEXA_OP_FORM=1) is bounded.
    With HEXA_OP_TEST_STALL=q, CTA 0 leaves out its layer load q, so its threads'
    wait for that layer runs out (about half a second of clock cycles): the
    kernel sets its error word, drains its other copies and returns, and the
    call reports HEXA_ERR_CUDA with the reason.  The context stays usable: an
    FP64 apply (no staging) afterwards is correct.  Runs in a child process
    because the variable is read once per process."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = str(Path(__file__).resolve().parents[1])
    script = f"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
from oracle import reference as ref
from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.solver import apply_operator
ctx = _lib.Context(0)
g = _lib.make_grid(40, 20, 20)
rng = np.random.default_rng(0)
fac = rng.uniform(0.1, 1, 40 * 20 * 20)
x = rng.standard_normal(3 * 41 * 21 * 21)
try:
    apply_operator(g, fac.astype(np.float32), x.astype(np.float32), clamp_faces=1, ctx=ctx, fp32=True)
    print("NO_ERROR")
except _lib.HexaError as e:
    print("ERR", e.code, str(e))
y = apply_operator(g, fac, x, clamp_faces=1, ctx=ctx)
gg = ref.Grid(40, 20, 20)
y_ref = ref.apply_A(gg, ref.canonical_stiffness(1, 1, 1, 0.3), fac, x, ref.fixed_mask(gg, 1))
print("FP64_ERR", float(np.abs(y - y_ref).max() / np.abs(y_ref).max()))
"""
    env = dict(os.environ, HEXA_OP_TEST_STALL="5", HEXA_OP_FORM="1")  # the TMA-staged form
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "ERR -2" in r.stdout and "bounded wait ran out" in r.stdout, r.stdout
    err = float(r.stdout.split("FP64_ERR")[1].split()[0])
    assert err < 1e-13


def test_staged_operator_form_matches_oracle():
    """The TMA-staged FP32 form (HEXA_OP_FORM=1, an alternative to the default
    one-row form) against the oracle on grids with boundary and interior
    tiles, every operator mode it serves through the solver included (a
    multigrid solve).  Child process: the form is read once per process."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = str(Path(__file__).resolve().parents[1])
    script = f"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
from oracle import reference as ref
from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads
from v119_2025_12_19_hexatop_aws_gb300.solver import apply_operator, solve
ctx = _lib.Context(0)
rng = np.random.default_rng(3)
worst = 0.0
for dims in [(5, 3, 7), (33, 17, 9), (62, 15, 20), (64, 32, 12)]:
    g = ref.Grid(*dims)
    fac = rng.uniform(1e-3, 1.0, g.nelem).astype(np.float32)
    x = rng.standard_normal(g.ndof).astype(np.float32)
    fixed = ref.fixed_mask(g, 1)
    y_ref = ref.apply_A(g, ref.canonical_stiffness(1, 1, 1, 0.3), fac.astype(np.float64), x.astype(np.float64), fixed)
    y = apply_operator(_lib.make_grid(*dims), fac, x, clamp_faces=1, ctx=ctx, fp32=True)
    worst = max(worst, float(np.abs(y - y_ref).max() / np.abs(y_ref).max()))
print("OP_ERR", worst)
dims = (16, 8, 8)
g = ref.Grid(*dims)
fac = rng.uniform(0.1, 1.0, g.nelem)
f = workloads.edge_load(*dims)
fixed = ref.fixed_mask(g, 1)
K0 = ref.canonical_stiffness(1, 1, 1, 0.3)
u_ref = ref.direct_solve(g, K0, fac, f, fixed, 0.0)
u, st = solve(_lib.make_grid(*dims), fac, f, clamp_faces=1, ctx=ctx,
              params=_lib.default_params(precision="mixed", tol=1e-12, max_iter=20000, mg_levels=3, shift_factor=0.0))
print("SOLVE_ERR", float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)), st["status"])
"""
    env = dict(os.environ, HEXA_OP_FORM="1")
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    op_err = float(r.stdout.split("OP_ERR")[1].split()[0])
    solve_err, status = r.stdout.split("SOLVE_ERR")[1].split()[:2]
    assert op_err <= 2e-6
    assert float(solve_err) <= 1e-9 and int(status) == 0
