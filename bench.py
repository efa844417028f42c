#!/usr/bin/env python
"""Benchmark of the FE-solve path on the seeded cantilever workloads.

One step = one solve of K_ff u = f to FP64 relative residual
||f - K u|| / ||f|| <= 1e-9 (recomputed in FP64) on the 384x192x192
cantilever (c3, 43,022,595 DOF) by the mixed-precision form: FP32 GMG-PCG
(autotuned levels and Chebyshev smoothing) inside FP64 reliable updates,
CUDA-graph replayed.  The line also carries the plain FP64 GMG-PCG solve of
the same system, the same mixed solve of the reference's shifted system
(K_ff + sigma I, sigma = 1e-10 max diag), the live roofline of the dominant
kernel (the FP32 operator's Chebyshev step) and the CPU baseline (the
reference's CPUSolver.jl path restated, Float32 Jacobi-PCG on all host cores).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--config c3|c2|c1|c4|c5]

Inputs are resident in HBM for ``value``; ``e2e`` repeats the step through the
C ABI with pinned host buffers (copies inside the timed region).  Inputs
(factor 113 MB, f and u 344 MB each at c3) exceed the 129 MB L2, so no
explicit flush is done between steps.  --config c2 times the plain FP64 form
(4-level GMG V(2,2) damped-Jacobi PCG) with the filter and the sensitivities.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "solve s to FP64 rel.res 1e-9, mixed vs plain FP64 on 1 GB300; matvec HBM GB/s"
FALLBACK_HBM_GBS = 6800.0
JACOBI_ITERS_FILE = ROOT / "profiles" / "jacobi_iterations.json"
TRAFFIC_FILE = ROOT / "profiles" / "op_traffic.json"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c1-c3: one cantilever solve; c4: 8 load cases on the c2 grid as one block PCG; "
                         "c5: 64 uneven cantilevers (filter + solve) as one batch")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: the warm-up and timed mixed steps only (no plain FP64, e2e, roofline or "
                         "CPU legs), the timed steps bracketed by cudaProfilerStart/Stop for "
                         "ncu --profile-from-start off; used for the launch lists under profiles/")
    ap.add_argument("--mg", default=None,
                    help="levels,steps,ratio: fixed multigrid settings for the mixed solves instead of the "
                         "autotuner (profile runs, where ncu's own overhead would distort the tuner's timings)")
    ap.add_argument("--count-jacobi", action="store_true",
                    help="count the iterations a FP64 Jacobi-PCG (every iteration tested, no shift) needs to reach "
                         "true rel.res 1e-9 on the config's system and print them as JSON (the record the CPU "
                         "baseline's projection uses, profiles/jacobi_iterations.json)")
    ap.add_argument("--kernel", default=None, choices=["apply", "apply_dot", "residual", "jacobi", "chebyshev",
                                                       "apply_fp64"],
                    help="time one operator mode alone on the config grid (--steps launches after --warmup) and "
                         "print its GB/s; the small case for ncu --set full captures")
    return ap.parse_args()


# --------------------------------------------------------------------- env
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, backend):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group(backend)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [l.split(", ") for l in Path(self.f.name).read_text().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------- workload
def workload(name):
    from v119_2025_12_19_hexatop_aws_gb300 import workloads as W
    nx, ny, nz = W.SIZES[name]
    return nx, ny, nz


def bench_config(name, ws):
    """The workload both arms measure (the same dict in both JSON lines)."""
    nx, ny, nz = workload(name)
    ndof = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    dens = ("seeded density 0.3+U(-0.05,0.05)" if name == "c1" else
            "seeded Gaussian density smoothed by the Helmholtz filter (r=4 elements), clamped to [0.001,1], mean 0.3")
    what = ("one FP64 solve + density filter (r=1.5) + sensitivities" if name == "c2" else "one solve")
    return {"workload": f"{name} cantilever {nx}x{ny}x{nz} hex8 ({ndof} DOF), x=0 clamped, unit -z load on the "
                        f"x=max,z=0 edge, SIMP p=3 E0=1 Emin=1e-9 nu=0.3, {dens}; step = {what} of K_ff u = f "
                        f"to FP64 ||f-Ku||/||f|| <= 1e-9",
            "parallelism": f"replicas{ws}", "l2": "inputs larger than L2 (no flush)"}


def _finish_inputs(name, rho):
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads as W
    nx, ny, nz = workload(name)
    fac = W.EMIN + rho ** W.PENAL * (W.E0 - W.EMIN)
    return _lib.make_grid(nx, ny, nz), rho, fac, W.edge_load(nx, ny, nz)


def make_inputs(name, ctx):
    """Seeded cantilever inputs (host numpy).  The c2/c3 density is smoothed by
    this library's GPU Helmholtz filter (FP64, tol 1e-10; input generation,
    outside any timed region)."""
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads as W
    from v119_2025_12_19_hexatop_aws_gb300.helmholtz import filter_density
    nx, ny, nz = workload(name)
    grid = _lib.make_grid(nx, ny, nz)
    if name == "c1":
        rho = W.c1_density(nx, ny, nz)
    else:
        def filt(g, R):
            out, _ = filter_density(grid, np.ascontiguousarray(g), R, tol=1e-10, max_iter=20000, quirk=False, ctx=ctx)
            return out
        rho = W.smooth_density(nx, ny, nz, filt)
    return _finish_inputs(name, rho)


def make_inputs_host(name):
    """The same inputs made on the host for the reference arm: the filter is the
    oracle's C restatement of the reference's Jacobi-PCG filter loop (FP64, tol
    1e-10), so this arm loads nothing of this library.  The densities agree
    with make_inputs' to about the filter tolerance."""
    from oracle import reference as ref
    from v119_2025_12_19_hexatop_aws_gb300 import workloads as W
    nx, ny, nz = workload(name)
    if name == "c1":
        rho = W.c1_density(nx, ny, nz)
    else:
        g = ref.Grid(nx, ny, nz)

        def filt(x, R):
            out, _, _ = ref.helmholtz_pcg_c(g, x, R, 1e-10, max_iter=20000, quirk=False)
            return out
        rho = W.smooth_density(nx, ny, nz, filt)
    return _finish_inputs(name, rho)


MG_OVERRIDE = None


def solver_params(name, precision, shift_factor=0.0):
    """The benchmarked system is the unshifted K_ff u = f (shift_factor 0);
    shift_factor 1e-10 gives the reference's (K_ff + sigma I) u = f.  The plain
    FP64 form uses the configuration's multigrid (4 levels and damped-Jacobi
    V(2,2) at c2; 5 levels and Chebyshev V(2,2) at c3); the mixed form is the
    autotuned one (level count and Chebyshev steps picked by trial solves on
    the first call, then cached)."""
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads as W
    # the reference's rel > 10 divergence stop (GPUSolver.jl:397) is off: CG residuals of these
    # high-contrast systems oscillate above it on the way to convergence
    if precision == "mixed" and MG_OVERRIDE:
        lv, nu, ratio = MG_OVERRIDE
        return _lib.default_params(precision=precision, precond="multigrid", tol=1e-9, max_iter=60000, mg_levels=lv,
                                   pre_smooth=nu, post_smooth=nu, cheb_ratio=ratio, divergence_check=0, autotune=0,
                                   shift_factor=shift_factor)
    extra = {"smoother": "jacobi"} if (name == "c2" and precision == "fp64") else {}
    return _lib.default_params(precision=precision, precond="multigrid", tol=1e-9, max_iter=60000,
                               mg_levels=W.MG_LEVELS.get(name, 0), pre_smooth=2, post_smooth=2,
                               divergence_check=0, autotune=1 if precision == "mixed" else 0,
                               shift_factor=shift_factor, **extra)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------ CPU baseline
def cpu_sample(name, fac, f, seconds, clamp_faces=1):
    """CPUSolver.jl's Float32 Jacobi-PCG on all host cores, on the unshifted
    system (solver_parameters.diagonal_shift_factor = 0, min_stiffness_threshold
    = 0 so that no element is skipped), a bounded number of
    iterations on the full grid; projected to a full solve with the iteration
    count a Jacobi-PCG needs for this system (counted once in FP64 to a true
    residual <= 1e-9 and recorded in profiles/jacobi_iterations.json).  A
    sample that converges (c1) is a measured full solve."""
    from oracle import reference as ref
    nx, ny, nz = workload(name)
    g = ref.Grid(nx, ny, nz)
    fixed = ref.fixed_mask(g, clamp_faces).astype(np.uint8)
    dens = fac.astype(np.float32)  # E = 1: density argument = modulus factor
    rec = {}
    if JACOBI_ITERS_FILE.exists():
        rec = json.loads(JACOBI_ITERS_FILE.read_text()).get(name, {})
    iters_needed = rec.get("iterations") if rec.get("true_relres", 1.0) <= 1e-9 else None
    # every element stays in the operator (min_stiffness_threshold 0: the factors reach down to Emin), so the
    # CPU path applies the same K_ff as the GPU
    _, rel, it, sec = ref.cpu_matrix_free_cg(g, 1.0, dens, f.astype(np.float32), fixed, nu=0.3,
                                             min_stiffness_threshold=0.0, max_iter=100000, tol=1e-9,
                                             shift_factor=0.0, max_seconds=seconds)
    per_iter = sec / max(it, 1)
    cores = ref.num_threads()
    if rel <= 1e-9:  # the sample ran to convergence: a measured full solve
        return {"value": sec, "unit": "s", "cores": cores, "kind": "port", "projected": False,
                "sample": f"a full Float32 Jacobi-PCG solve of CPUSolver.jl's matrix_free path on the {nx}x{ny}x{nz} "
                          f"grid ({it} iterations to rel.res {rel:.2e}, {per_iter:.4f} s/iteration)",
                "s_per_iteration": per_iter, "timed_iterations": it}
    if iters_needed:
        value = per_iter * iters_needed
        sample = (f"{it} Float32 Jacobi-PCG iterations of CPUSolver.jl's matrix_free path on the full {nx}x{ny}x{nz} "
                  f"grid timed ({sec:.1f} s, {per_iter:.3f} s/iteration) x {iters_needed} iterations that a "
                  f"Jacobi-PCG needs to reach true rel.res 1e-9 on this system (counted once in FP64, "
                  f"{JACOBI_ITERS_FILE.name})")
    else:
        value = None
        sample = f"{it} iterations, {per_iter:.3f} s/iteration; Jacobi iteration count to 1e-9 not recorded"
    return {"value": value, "unit": "s", "cores": cores, "kind": "port", "projected": True, "sample": sample,
            "s_per_iteration": per_iter, "timed_iterations": it, "projected_iterations": iters_needed}


# -------------------------------------------------------------- our arm
def run_ours(a):
    import torch
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads as W
    from v119_2025_12_19_hexatop_aws_gb300 import build as libbuild
    import ctypes as C

    libbuild.build()
    dist = Dist("nccl")
    torch.cuda.set_device(dist.local)
    ctx = _lib.Context(dist.local)
    grid, rho, fac, f = make_inputs(a.config, ctx)
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    ndof, nelem = 3 * (nx + 1) * (ny + 1) * (nz + 1), nx * ny * nz
    dev = torch.device("cuda", dist.local)
    fac_d = torch.from_numpy(fac).to(dev)
    f_d = torch.from_numpy(f).to(dev)
    u_d = torch.empty(ndof, dtype=torch.float64, device=dev)
    rho_d = torch.from_numpy(rho).to(dev)
    filt_d = torch.empty_like(rho_d)
    dc_d = torch.empty_like(rho_d)
    bc = _lib.make_bc(1)
    plain_step = a.config == "c2"  # c2: the plain FP64 form is the step
    pm = solver_params(a.config, "fp64" if plain_step else "mixed")
    st = _lib.SolveStats()
    fst = _lib.FilterStats()
    cval = C.c_double()

    def solve(params, fac_p, f_p, u_p):
        rc = ctx.lib.hexa_solve(ctx.h, C.byref(grid), C.byref(bc), fac_p, f_p, C.byref(params), None, u_p,
                                C.byref(st))
        ctx.check(rc, allow=(_lib.HEXA_OK,))
        return st.as_dict()

    def filt():  # the SIMP step's density filter, r = 1.5 elements (FP64)
        ctx.check(ctx.lib.hexa_filter(ctx.h, C.byref(grid), rho_d.data_ptr(), W.helmholtz_R(1.5), 1e-5, 200, 1, 0,
                                      filt_d.data_ptr(), C.byref(fst)), allow=(_lib.HEXA_OK,))

    def sens():
        ctx.check(ctx.lib.hexa_sensitivities(ctx.h, C.byref(grid), 0.3, rho_d.data_ptr(), u_d.data_ptr(), W.EMIN,
                                             W.E0, W.PENAL, dc_d.data_ptr(), C.byref(cval)), allow=(_lib.HEXA_OK,))

    def step(fac_p, f_p, u_p):
        out = solve(pm, fac_p, f_p, u_p)
        if plain_step:
            filt()
            sens()
        return out

    if a.kernel:
        run_kernel(a, ctx, grid, bc, fac_d, f_d, ndof, nelem, dist)
        return

    first = None
    for w in range(a.warmup):
        t_first = time.perf_counter()
        sw = step(fac_d.data_ptr(), f_d.data_ptr(), u_d.data_ptr())
        if w == 0:  # the first call on a grid pays the hierarchy set-up and, mixed, the autotuner's trial solves
            torch.cuda.synchronize()
            first = {"wall_s": round(time.perf_counter() - t_first, 4), "setup_ms": sw["setup_ms"],
                     "solve_ms": sw["solve_ms"]}
    torch.cuda.synchronize()
    dist.barrier()
    clocks = Clocks(dist.local)
    clocks.start()
    l0 = ctx.kernel_launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if a.profile:
        torch.cuda.profiler.start()
    ev0.record()
    stats = []
    for _ in range(a.steps):
        stats.append(step(fac_d.data_ptr(), f_d.data_ptr(), u_d.data_ptr()))
    ev1.record()
    torch.cuda.synchronize()
    if a.profile:
        torch.cuda.profiler.stop()
    ck = clocks.stop()
    dist.barrier()
    launches = ctx.kernel_launches - l0
    ms = ev0.elapsed_time(ev1) / a.steps
    ms = dist.max(ms)
    s_last = stats[-1]
    comp_step = s_last["compliance"]

    if a.profile:
        if dist.rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(ms / 1e3, 6), "unit": "s", "profile_run": True,
                              "steps": a.steps, "warmup": a.warmup, "iterations": s_last["iterations"],
                              "mg_levels": s_last["mg_levels"], "smooth_steps": s_last["smooth_steps"],
                              "gpu_launches": int(launches)}))
        ctx.close()
        dist.close()
        return

    def timed_once(params, u_out):
        """One solve after an allocating call (one iteration per attempt), timed alone."""
        pre = _lib.SolveParams.from_buffer_copy(params)
        pre.max_iter, pre.max_shift_attempts = 1, 1
        ctx.check(ctx.lib.hexa_solve(ctx.h, C.byref(grid), C.byref(bc), fac_d.data_ptr(), f_d.data_ptr(),
                                     C.byref(pre), None, u_out.data_ptr(), C.byref(st)),
                  allow=(_lib.HEXA_OK, _lib.HEXA_NOT_CONVERGED))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        so = solve(params, fac_d.data_ptr(), f_d.data_ptr(), u_out.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), so

    def dc_of(u):
        dc = torch.empty_like(rho_d)
        cv = C.c_double()
        ctx.check(ctx.lib.hexa_sensitivities(ctx.h, C.byref(grid), 0.3, rho_d.data_ptr(), u.data_ptr(), W.EMIN,
                                             W.E0, W.PENAL, dc.data_ptr(), C.byref(cv)), allow=(_lib.HEXA_OK,))
        return dc

    def rel_diffs(u_a, comp_a, u_b, comp_b):
        out = {"compliance_rel_diff": abs(comp_a - comp_b) / abs(comp_b),
               "u_rel_diff": (torch.linalg.vector_norm(u_a - u_b) / torch.linalg.vector_norm(u_b)).item()}
        try:
            da, db = dc_of(u_a), dc_of(u_b)
            out["dc_rel_diff"] = (torch.linalg.vector_norm(da - db) / torch.linalg.vector_norm(db)).item()
        except Exception as e:  # never voids the line
            out["dc_rel_diff"] = f"error: {e}"[:160]
        return out

    # the other form of the same unshifted system: plain FP64 beside the mixed step, or mixed beside the plain c2 step
    other = None
    if not a.no_plain:
        if plain_step:
            om, so = timed_once(solver_params(a.config, "mixed"), torch.empty_like(u_d))
            other = {"form": "mixed", "s": om / 1e3, "iterations": so["iterations"],
                     "unshifted_relres": so["unshifted_relres"], "compliance": so["compliance"]}
        else:
            u64 = torch.empty_like(u_d)
            pms, sp = timed_once(solver_params(a.config, "fp64"), u64)
            other = {"form": "plain FP64 GMG-PCG", "s": pms / 1e3, "iterations": sp["iterations"],
                     "unshifted_relres": sp["unshifted_relres"], "compliance": sp["compliance"],
                     "mixed_over_plain": ms / pms}
            other.update({k + "_mixed": v for k, v in rel_diffs(u_d, comp_step, u64, sp["compliance"]).items()})
            del u64

    # the reference's shifted system (K_ff + sigma I) u = f, sigma = 1e-10 max diag (GPUSolver.jl:343)
    shifted = None
    if not a.no_plain and not plain_step:
        us = torch.empty_like(u_d)
        sms, ss = timed_once(solver_params(a.config, "mixed", shift_factor=1e-10), us)
        shifted = {"s": sms / 1e3, "iterations": ss["iterations"], "sigma": ss["shift"],
                   "shifted_true_relres": ss["true_relres"], "unshifted_relres": ss["unshifted_relres"],
                   "compliance": ss["compliance"],
                   "compliance_rel_diff_to_unshifted": abs(ss["compliance"] - comp_step) / abs(comp_step)}
        del us

    # e2e: the same step through the C ABI with pinned host buffers
    fac_h = torch.from_numpy(fac).pin_memory()
    f_h = torch.from_numpy(f).pin_memory()
    u_h = torch.empty(ndof, dtype=torch.float64).pin_memory()
    step(fac_h.data_ptr(), f_h.data_ptr(), u_h.data_ptr())
    ke = max(1, min(a.steps, 3))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(ke):
        step(fac_h.data_ptr(), f_h.data_ptr(), u_h.data_ptr())
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = dist.max(e0.elapsed_time(e1) / ke)

    # roofline: the operator, each mode timed alone with CUDA events on the library's stream
    peak, peak_kind = peaks()
    f32 = lambda t: t.to(torch.float32).contiguous()
    facf, xf, bf = f32(fac_d), f32(u_d), f32(f_d)
    yf = torch.empty_like(xf)
    modes = {"apply": (0, 8 * ndof + 4 * nelem), "apply_dot": (1, 8 * ndof + 4 * nelem),
             "residual": (2, 12 * ndof + 4 * nelem), "jacobi": (4, 12 * ndof + 4 * nelem),
             "chebyshev": (5, 16 * ndof + 4 * nelem)}
    kern = {}
    for name, (mode, nbytes) in modes.items():
        t = C.c_double()
        yf.copy_(xf)  # the Chebyshev step runs in place over its previous iterate
        rc = ctx.lib.hexa_time_operator(ctx.h, C.byref(grid), C.byref(bc), 0.3, 2, mode, facf.data_ptr(),
                                        xf.data_ptr(), bf.data_ptr(), yf.data_ptr(), 20, C.byref(t))
        ctx.check(rc, allow=(_lib.HEXA_OK,))
        kern[name] = {"ms": t.value, "bytes": nbytes, "gbs": nbytes / (t.value * 1e-3) / 1e9}
    y64 = torch.empty_like(u_d)
    for name, mode, nbytes in (("apply_fp64", 0, 16 * ndof + 8 * nelem), ("chebyshev_fp64", 5, 32 * ndof + 8 * nelem)):
        t64 = C.c_double()
        y64.copy_(u_d)
        ctx.check(ctx.lib.hexa_time_operator(ctx.h, C.byref(grid), C.byref(bc), 0.3, 0, mode, fac_d.data_ptr(),
                                             u_d.data_ptr(), f_d.data_ptr(), y64.data_ptr(), 5, C.byref(t64)),
                  allow=(_lib.HEXA_OK,))
        kern[name] = {"ms": t64.value, "bytes": nbytes, "gbs": nbytes / (t64.value * 1e-3) / 1e9}
    del y64
    dom = kern["chebyshev_fp64" if plain_step else "chebyshev"]
    traffic = None
    if TRAFFIC_FILE.exists():
        key = "cheb2_fp64_bytes_per_launch" if plain_step else "cheb2_fp32_bytes_per_launch"
        traffic = json.loads(TRAFFIC_FILE.read_text()).get(a.config, {}).get(key)
    roof = {"bound": "hbm", "achieved": round(dom["gbs"], 1), "peak": peak, "unit": "GB/s",
            "frac": round(dom["gbs"] / peak, 4), "traffic": traffic,
            "kernel": "op_kernel<double, OP_CHEB2>" if plain_step else "op_kernel<float, OP_CHEB2>",
            "peak_source": peak_kind, "algorithmic_bytes_per_launch": dom["bytes"],
            "kernel_ms": round(dom["ms"], 5)}
    if plain_step:
        roof["note"] = "FP64 form: bound by GB300's FP64 issue rate, not by HBM"

    cpu = None
    if dist.rank == 0 and not a.no_cpu:
        cpu = cpu_sample(a.config, fac, f, a.cpu_seconds)

    # the SIMP step around the solve: density filter (r = 1.5 elements) and the
    # sensitivities of the solution, each timed with CUDA events
    pipe = {}
    for name, fn in (("filter_s", filt), ("sensitivities_s", sens)):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            fn()
        e1.record()
        torch.cuda.synchronize()
        pipe[name] = round(e0.elapsed_time(e1) / 3 / 1e3, 6)
    pipe["filter_iterations"] = int(fst.iterations)
    if not plain_step:
        pipe["solve_filter_sensitivities_s"] = round(ms / 1e3 + pipe["filter_s"] + pipe["sensitivities_s"], 6)

    try:
        rows = next_rows(ctx, grid, u_d, rho, dev, peak)
    except Exception as e:  # the rows either side of the solve never void the headline line
        rows = {"error": str(e)[:200]}

    dofit = ndof * s_last["iterations"] / (ms / 1e3)
    if plain_step:
        solver = (f"plain FP64 GMG-PCG ({s_last['mg_levels']} levels, damped-Jacobi V({s_last['smooth_steps']},"
                  f"{s_last['smooth_steps']})), then the FP64 density filter and the sensitivities")
    else:
        solver = (f"mixed: FP32 GMG-PCG (autotuned: {s_last['mg_levels']} levels, Chebyshev "
                  f"V({s_last['smooth_steps']},{s_last['smooth_steps']}) on [lmax/{pm.cheb_ratio}, lmax]) with FP64 "
                  f"reliable updates to true residual 1e-9; beside it plain FP64 GMG-PCG "
                  f"({solver_params(a.config, 'fp64').mg_levels} levels, V(2,2))")
    out = {
        "metric": METRIC, "value": round(ms / 1e3, 6), "unit": "s", "n_gpus": dist.ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if plain_step else "f32+f64",
        "data": "synthetic (seeded cantilever, Helmholtz-smoothed density)",
        "config": bench_config(a.config, dist.ws),
        "solver": solver,
        "parity": "partial: the oracle restates the reference's path; the reference (Julia) ships no tests or fixtures "
                  "and cannot run here, so parity with it is unpinned beyond exact element-matrix KATs",
        "e2e": {"value": round(e2e_ms / 1e3, 6), "unit": "s", "h2d_bytes_per_step": 8 * (nelem + ndof),
                "d2h_bytes_per_step": 8 * ndof},
        "roofline": roof,
        "cpu_baseline": cpu,
        "gpu_launches": int(launches),
        "clocks": ck,
        "solve": {"iterations": s_last["iterations"], "outer_iterations": s_last["outer_iterations"],
                  "mg_levels": s_last["mg_levels"], "smooth_steps": s_last["smooth_steps"],
                  "shift": s_last["shift"], "unshifted_relres": s_last["unshifted_relres"],
                  "true_relres": s_last["true_relres"], "compliance": comp_step,
                  "fine_applies": s_last["fine_applies"], "dof_iterations_per_s": dofit,
                  "setup_ms": s_last["setup_ms"], "solve_ms": s_last["solve_ms"],
                  "first_call": first},
        "other_form": other,
        "reference_shifted_system": shifted,
        "simp_step": pipe,
        "kernels": kern,
        "next_rows": rows,
    }
    if dist.rank == 0:
        print(json.dumps(out))
    ctx.close()
    dist.close()


def next_rows(ctx, grid, u_d, rho, dev, peak=None, reps=3):
    """The kernels either side of the solve on the solved workload, device
    arrays, each timed over `reps` calls after one warm call (the calls end
    with a stream synchronize, so the events bracket complete work):
    stress post-processing of the mixed solution, the density update with and
    without its filter, and the refiner transfer onto a grid with 1.2x the
    elements.  Algorithmic bytes: stress 48 B/element (density in; principal
    stresses, directions, von Mises, L1 out) + 24 B/node (displacements);
    update without filter 28 B/element (proposal 8, update 12, finish 8);
    remap 12 B per new element (8 out + about 4 in)."""
    import ctypes as C
    import torch
    from v119_2025_12_19_hexatop_aws_gb300 import _lib
    from v119_2025_12_19_hexatop_aws_gb300.refine import element_distribution
    from v119_2025_12_19_hexatop_aws_gb300.topopt import density_update_params
    ne = grid.nx * grid.ny * grid.nz
    nn = (grid.nx + 1) * (grid.ny + 1) * (grid.nz + 1)
    dens = torch.from_numpy(np.asarray(rho, dtype=np.float32)).to(dev)
    outs = [torch.empty(3 * ne, dtype=torch.float32, device=dev) for _ in range(3)]
    vm, l1 = torch.empty(ne, dtype=torch.float32, device=dev), torch.empty(ne, dtype=torch.float32, device=dev)
    ok = (_lib.HEXA_OK,)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def stress():
        ctx.check(ctx.lib.hexa_stress_field(ctx.h, C.byref(grid), u_d.data_ptr(), dens.data_ptr(), 1.0, 0.3,
                                            outs[0].data_ptr(), vm.data_ptr(), None, l1.data_ptr(),
                                            outs[1].data_ptr(), outs[2].data_ptr()), allow=ok)

    rows = {}
    t = timed(stress)
    b = 48 * ne + 24 * nn
    rows["stress"] = {"ms": round(t, 4), "bytes": b, "gbs": round(b / (t * 1e-3) / 1e9, 1)}
    allow = float(l1.max().item()) / 2.0 or 1.0
    orig = torch.ones(ne, dtype=torch.float32, device=dev)
    work = torch.empty_like(dens)
    st = _lib.DensityUpdateStats()
    for name, kw in (("update_no_filter", {"minimum_filter_radius_as_elements": 0.0}), ("update", {})):
        prm = density_update_params(E=1.0, l1_stress_allowable=allow, iter=10, number_of_iterations=30,
                                    max_domain_dim=float(max(grid.nx * grid.dx, grid.ny * grid.dy, grid.nz * grid.dz)),
                                    **kw)

        def upd():
            work.copy_(dens)
            ctx.check(ctx.lib.hexa_update_density(ctx.h, C.byref(grid), work.data_ptr(), l1.data_ptr(), None,
                                                  orig.data_ptr(), C.byref(prm), C.byref(st)), allow=ok)

        t = timed(upd)
        rows[name] = {"ms": round(t, 4), "culled": int(st.culled), "filter_iters": int(st.filter_iters)}
        if name == "update_no_filter":
            rows[name].update(bytes=28 * ne, gbs=round(28 * ne / (t * 1e-3) / 1e9, 1))
    L = (grid.nx * grid.dx, grid.ny * grid.dy, grid.nz * grid.dz)
    nx, ny, nz, dx, dy, dz, cnt = element_distribution(*L, int(ne * 1.2))
    ng = _lib.make_grid(nx, ny, nz, dx, dy, dz)
    nd, na = torch.empty(cnt, dtype=torch.float32, device=dev), torch.empty(cnt, dtype=torch.float32, device=dev)

    def remap():
        ctx.check(ctx.lib.hexa_remap_fields(ctx.h, C.byref(grid), C.byref(ng), *[float(np.float32(v)) for v in L],
                                            dens.data_ptr(), orig.data_ptr(), 1, nd.data_ptr(), na.data_ptr()),
                  allow=ok)

    t = timed(remap)
    rows["remap"] = {"ms": round(t, 4), "new_grid": [nx, ny, nz], "bytes": 12 * cnt,
                     "gbs": round(12 * cnt / (t * 1e-3) / 1e9, 1)}
    if peak:
        for r in rows.values():
            if "gbs" in r:
                r["frac_of_measured_hbm"] = round(r["gbs"] / peak, 4)
    return rows


OP_MODES = {"apply": (0, 2, 8, 4), "apply_dot": (1, 2, 8, 4), "residual": (2, 2, 12, 4), "jacobi": (4, 2, 12, 4),
            "chebyshev": (5, 2, 16, 4), "apply_fp64": (0, 0, 16, 8)}  # mode, precision, B/DOF, B/element


def run_kernel(a, ctx, grid, bc, fac_d, f_d, ndof, nelem, dist):
    """One operator mode alone: --warmup launches, then --steps launches timed
    by the library with CUDA events on its stream (algorithmic bytes: B/DOF * nDOF
    + B/element * nElem per launch)."""
    import ctypes as C
    import torch
    from v119_2025_12_19_hexatop_aws_gb300 import _lib

    mode, prec, bdof, belem = OP_MODES[a.kernel]
    cast = (lambda t: t.to(torch.float32).contiguous()) if prec == 2 else (lambda t: t)
    fac, x, b = cast(fac_d), cast(torch.rand_like(f_d)), cast(f_d)
    y = torch.empty_like(x)
    t = C.c_double()
    for reps in (max(1, a.warmup), max(1, a.steps)):
        ctx.check(ctx.lib.hexa_time_operator(ctx.h, C.byref(grid), C.byref(bc), 0.3, prec, mode, fac.data_ptr(),
                                             x.data_ptr(), b.data_ptr(), y.data_ptr(), reps, C.byref(t)),
                  allow=(_lib.HEXA_OK,))
    nbytes = bdof * ndof + belem * nelem
    peak, kind = peaks()
    if dist.rank == 0:
        print(json.dumps({"kernel": a.kernel, "config": a.config, "ms_per_launch": t.value,
                          "algorithmic_bytes": nbytes, "gbs": nbytes / (t.value * 1e-3) / 1e9,
                          "frac": nbytes / (t.value * 1e-3) / 1e9 / peak, "peak": peak, "peak_source": kind,
                          "launches": max(1, a.warmup) + max(1, a.steps)}))
    ctx.close()
    dist.close()


# -------------------------------------------------------- reference arm
def run_reference(a):
    """The reference's own CPU path for this solve (CPUSolver.jl restated, the
    oracle port; the reference is Julia and cannot run here), timed on the
    host cores on bounded samples of the same workload.  Inputs are made on
    the host by the oracle (make_inputs_host): this arm loads nothing of this
    library.  The value is a projection (timed iterations x the iteration count
    a Jacobi-PCG needs), labelled as such."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from oracle import build as obuild
    obuild.build()
    name = a.config if a.config in ("c1", "c2", "c3") else "c3"
    grid, rho, fac, f = make_inputs_host(name)
    per_step = max(2.0, a.cpu_seconds / 2)
    vals, last = [], None
    for i in range(a.warmup + a.steps):
        r = cpu_sample(name, fac, f, per_step)
        if i >= a.warmup:
            vals.append(r["value"] if r["value"] is not None else float("nan"))
            last = r
    v = float(np.mean(vals))
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded cantilever, Helmholtz-smoothed density)",
        "config": bench_config(name, ws),
        "solver": "reference CPU matrix_free path (CPUSolver.jl restated): Float32 Jacobi-PCG on all host cores, "
                  "every element kept, no diagonal shift",
        "projected": bool(last.get("projected")),
        "cpu_baseline": {**last, "value": v},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_count_jacobi(a):
    """FP64 Jacobi-PCG of the config's unshifted system, ||r||/||f|| tested
    every iteration as CPUSolver.jl does, continued until the FP64 true residual
    is <= 1e-9; prints the iteration count."""
    import ctypes as C
    import torch
    from v119_2025_12_19_hexatop_aws_gb300 import _lib
    from v119_2025_12_19_hexatop_aws_gb300 import build as libbuild
    libbuild.build()
    ctx = _lib.Context(0)
    grid, rho, fac, f = make_inputs(a.config, ctx)
    fac_d, f_d = torch.from_numpy(fac).cuda(), torch.from_numpy(f).cuda()
    u_d = torch.empty_like(f_d)
    p = _lib.default_params(precision="fp64", precond="jacobi", tol=1e-9, max_iter=2000000, shift_factor=0.0,
                            check_cadence=1, divergence_check=0, max_shift_attempts=1, true_residual=1)
    st = _lib.SolveStats()
    t0 = time.perf_counter()
    rc = ctx.lib.hexa_solve(ctx.h, C.byref(grid), C.byref(_lib.make_bc(1)), fac_d.data_ptr(), f_d.data_ptr(),
                            C.byref(p), None, u_d.data_ptr(), C.byref(st))
    torch.cuda.synchronize()
    nx, ny, nz = workload(a.config)
    print(json.dumps({a.config: {"iterations": st.iterations, "grid": f"{nx}x{ny}x{nz}", "dof": 3 * (nx + 1) * (ny + 1) * (nz + 1),
                                 "recursive_relres": st.relres, "true_relres": st.true_relres,
                                 "unshifted_relres": st.unshifted_relres, "shift": st.shift, "status": rc,
                                 "gpu_solve_s": round(time.perf_counter() - t0, 2)}}))
    ctx.close()


# ------------------------------------------------------------- batching
def _timed(fn, warmup, steps):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = None
    for _ in range(steps):
        out = fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / steps, out


def run_c4(a):
    """k = 8 load cases on the c2 cantilever: one block PCG (FP32 inner, FP64
    reliable updates to 1e-9 per column) against 8 separate mixed solves."""
    import ctypes as C
    import torch
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads as W
    from v119_2025_12_19_hexatop_aws_gb300 import build as libbuild
    libbuild.build()
    ctx = _lib.Context(0)
    grid, rho, fac, _ = make_inputs("c2", ctx)
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    F = W.point_loads(nx, ny, nz, 8)
    k, ndof = F.shape
    fac_d = torch.from_numpy(fac).cuda()
    F_d = torch.from_numpy(F).cuda()
    U_d = torch.empty_like(F_d)
    u_d = torch.empty(ndof, dtype=torch.float64, device="cuda")
    bc = _lib.make_bc(1)
    pm = solver_params("c4", "mixed")
    st = _lib.SolveStats()

    def block():
        ctx.check(ctx.lib.hexa_solve_multi_rhs(ctx.h, C.byref(grid), C.byref(bc), fac_d.data_ptr(), k, F_d.data_ptr(),
                                               C.byref(pm), U_d.data_ptr(), C.byref(st)), allow=(_lib.HEXA_OK,))
        return st.as_dict()

    def columns():
        out = []
        for j in range(k):
            ctx.check(ctx.lib.hexa_solve(ctx.h, C.byref(grid), C.byref(bc), fac_d.data_ptr(), F_d[j].data_ptr(),
                                         C.byref(pm), None, u_d.data_ptr(), C.byref(st)), allow=(_lib.HEXA_OK,))
            out.append(st.as_dict())
        return out

    if a.profile:  # one block solve inside cudaProfilerStart/Stop, for ncu launch lists
        for _ in range(max(1, a.warmup)):
            block()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        sb = block()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"metric": "c4 block solve (profile run)", "iterations": sb["iterations"],
                          "solve_ms": sb["solve_ms"], "profile_run": True}))
        ctx.close()
        return
    tb, sb = _timed(block, a.warmup, a.steps)
    tc, sc = _timed(columns, 1, 1)
    print(json.dumps({"metric": "s per 8-load-case solve to FP64 rel.res 1e-9 per column", "value": round(tb, 4),
                      "unit": "s", "config": {"workload": f"c4 cantilever {nx}x{ny}x{nz}, {ndof} DOF, 8 point loads, "
                                                          "block PCG, FP32 inner / FP64 reliable updates"},
                      "steps": a.steps, "warmup": a.warmup, "block": sb,
                      "separate_mixed_solves_s": round(tc, 4), "separate_iterations": [q["iterations"] for q in sc],
                      "compliance_sum_block": sb["compliance"],
                      "compliance_sum_separate": sum(q["compliance"] for q in sc),
                      "block_over_separate": round(tb / tc, 4),
                      "ms_per_block_iteration": round(1e3 * tb / max(1, sb["iterations"]), 4),
                      "ms_per_single_rhs_iteration": round(1e3 * tc / max(1, sum(q["iterations"] for q in sc)), 4),
                      "block_iteration_over_single": round((tb / max(1, sb["iterations"])) /
                                                           (tc / max(1, sum(q["iterations"] for q in sc))), 3)}))
    ctx.close()


def run_c5(a):
    """64 uneven cantilevers: every instance's Helmholtz filter (r = 1.5) and
    mixed GMG-PCG solve as two batches, against the same work one instance at
    a time through the single-grid entry points."""
    import torch
    from v119_2025_12_19_hexatop_aws_gb300 import _lib, workloads as W
    from v119_2025_12_19_hexatop_aws_gb300 import build as libbuild
    from v119_2025_12_19_hexatop_aws_gb300.helmholtz import filter_batch, filter_density
    from v119_2025_12_19_hexatop_aws_gb300.solver import solve, solve_batch
    libbuild.build()
    ctx = _lib.Context(0)
    dims = W.batch_sizes(64)
    grids = [_lib.make_grid(*d) for d in dims]
    rhos, forces = [], []
    for i, (d, g) in enumerate(zip(dims, grids)):
        def filt(x, R, g=g):
            out, _ = filter_density(g, np.ascontiguousarray(x), R, tol=1e-10, max_iter=20000, quirk=False, ctx=ctx)
            return out
        rhos.append(W.smooth_density(*d, filt, seed=W.SEED + 1000 + i, r_elems=2.0))
        forces.append(W.point_loads(*d, 1, seed=W.SEED + 2000 + i)[0])
    rho_d = [torch.from_numpy(r).cuda() for r in rhos]
    f_d = [torch.from_numpy(f).cuda() for f in forces]
    filt_d = [torch.empty_like(r) for r in rho_d]
    u_d = [torch.empty_like(f) for f in f_d]
    R = W.helmholtz_R(1.5)
    pm = solver_params("c5", "mixed")

    # the in-batch filter runs the reference's loop (Jacobi-PCG, tolerance 1e-5, at most 200 iterations,
    # GPUHelmholtz.jl:190-266) in FP64: in FP32 the batched and the single-grid reductions, summed in
    # different orders, round differently and the two paths would not filter to the same densities
    filt_single = [torch.empty_like(r) for r in rho_d]

    def batch():
        filter_batch(grids, rho_d, R, tol=1e-5, max_iter=200, quirk=True, precision="fp64", out=filt_d, ctx=ctx)
        facs = [W.EMIN + r ** W.PENAL * (W.E0 - W.EMIN) for r in filt_d]
        _, st, rc = solve_batch(grids, facs, f_d, clamp_faces=1, params=pm, u_out=u_d, ctx=ctx)
        return st

    def one_by_one():
        st = []
        for i, g in enumerate(grids):
            fr, _ = filter_density(g, rho_d[i], R, tol=1e-5, max_iter=200, quirk=True, precision="fp64",
                                   out=filt_single[i], ctx=ctx)
            fac = W.EMIN + filt_single[i] ** W.PENAL * (W.E0 - W.EMIN)
            _, s = solve(g, fac, f_d[i], clamp_faces=1, params=pm, u_out=u_d[i], ctx=ctx)
            st.append(s)
        return st

    if a.profile:  # one batch (filter + solve) inside cudaProfilerStart/Stop
        for _ in range(max(1, a.warmup)):
            batch()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        sb = batch()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"metric": "c5 batch (profile run)", "iterations_max": max(s["iterations"] for s in sb),
                          "profile_run": True}))
        ctx.close()
        return
    tb, sb = _timed(batch, a.warmup, a.steps)
    comp_b = [s["compliance"] for s in sb]
    ts, ss = _timed(one_by_one, 1, 1)
    comp_s = [s["compliance"] for s in ss]
    nelem = sum(d[0] * d[1] * d[2] for d in dims)
    print(json.dumps({"metric": "s per batch of 64 uneven cantilevers (filter + solve to FP64 rel.res 1e-9)",
                      "value": round(tb, 4), "unit": "s", "steps": a.steps, "warmup": a.warmup,
                      "config": {"workload": f"c5: 64 cantilevers nx in 16..96 step 8, ny=nz=nx/2, "
                                             f"{nelem} elements in total, filter r=1.5, mixed GMG-PCG"},
                      "max_true_relres": max(s["true_relres"] for s in sb),
                      "iterations_max": max(s["iterations"] for s in sb),
                      "one_by_one_s": round(ts, 4), "batch_over_one_by_one": round(tb / ts, 4),
                      "max_rel_compliance_diff": max(abs(x - y) / abs(y) for x, y in zip(comp_b, comp_s)),
                      "max_abs_density_diff": max(float((a - b).abs().max()) for a, b in zip(filt_d, filt_single))}))
    ctx.close()


if __name__ == "__main__":
    args = parse()
    if args.mg:
        MG_OVERRIDE = tuple(int(v) for v in args.mg.split(","))
    if args.impl == "reference":
        run_reference(args)
    elif args.count_jacobi:
        run_count_jacobi(args)
    elif args.config == "c4":
        run_c4(args)
    elif args.config == "c5":
        run_c5(args)
    else:
        run_ours(args)
