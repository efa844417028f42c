"""Mesh growth between SIMP phases: the refinement decision and the field
transfer of MeshRefiner.refine_mesh_and_fields (src/Mesh/MeshRefiner.jl:77-243)
on the structured grid, the transfer itself on the GPU (hexa_remap_fields).

The decision restates the reference: the new total is the smallest of the
target-driven size (target_active / active_ratio * 0.9), the growth-rate
limit (n_old * max_growth_rate), the memory limit and the configured hard
limit; growth below 5 % is skipped; the new grid follows
Helpers.calculate_element_distribution (same element count per unit volume
in every direction).  The memory limit here is the GPU's free memory at 250 B
per element (the reference sizes host RAM the same way, MeshRefiner.jl:13-43).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .solver import context


def element_distribution(len_x, len_y, len_z, target):
    """Helpers.calculate_element_distribution (Utils/Helpers.jl:154-169) in
    Float32, the type of the reference's domain lengths (Float32 dx times the
    element count, Main.jl:273): (nx, ny, nz, dx, dy, dz, count)."""
    f32 = np.float32
    L = (f32(len_x), f32(len_y), f32(len_z))
    k = np.cbrt(f32(target) / (L[0] * L[1] * L[2]))
    n = [max(1, int(round(float(k * Li)))) for Li in L]
    h = [float(L[a] / f32(n[a])) for a in range(3)]
    return n[0], n[1], n[2], h[0], h[1], h[2], n[0] * n[1] * n[2]


@dataclass
class RefinePlan:
    refine: bool
    new_total: int
    limit: str


def plan_refinement(n_total_old, n_active_old, target_active, *, max_growth_rate=1.2, hard_element_limit=800_000_000,
                    memory_limit=None) -> RefinePlan:
    """The refinement decision of MeshRefiner.jl:101-146."""
    active_ratio = max(0.0001, n_active_old / n_total_old)
    if n_active_old >= target_active:
        return RefinePlan(False, n_total_old, "Target active count reached")
    limits = [("Target Active Limit", int(round(target_active / active_ratio * 0.90))),
              ("Growth Rate Limit", int(round(n_total_old * max_growth_rate))),
              ("RAM Limit", int(memory_limit if memory_limit is not None else hard_element_limit)),
              ("Config Hard Limit", int(hard_element_limit))]
    name, total = min(limits, key=lambda t: t[1])  # the first of equal limits, as a stable sort
    total = min(total, hard_element_limit)
    if total < n_total_old * 1.05:
        return RefinePlan(False, n_total_old, "growth below 5 %")
    return RefinePlan(True, total, name)


def domain_lengths(grid):
    """Float32 domain lengths dx * n as the reference forms them (Main.jl:273)."""
    f32 = np.float32
    return (float(f32(grid.dx) * f32(grid.nx)), float(f32(grid.dy) * f32(grid.ny)), float(f32(grid.dz) * f32(grid.nz)))


def gpu_memory_limit(bytes_per_element=250, safety=0.15):
    """Elements that fit the GPU's free memory after a safety margin."""
    import torch
    free, _ = torch.cuda.mem_get_info()
    return max(1_000_000, int(free * (1.0 - safety) / bytes_per_element))


def remap_fields(old_grid, new_grid, lengths, density, alpha=None, *, projection=True, ctx=None):
    """New-grid density (and alpha) by the GPU transfer; float32 arrays."""
    ctx = ctx or context()
    nn = new_grid.nx * new_grid.ny * new_grid.nz
    nd = np.empty(nn, np.float32)
    na = np.empty(nn, np.float32) if alpha is not None else None
    rc = ctx.lib.hexa_remap_fields(ctx.h, C.byref(old_grid), C.byref(new_grid), float(lengths[0]), float(lengths[1]),
                                   float(lengths[2]), _lib.ptr(np.ascontiguousarray(density, dtype=np.float32)),
                                   _lib.ptr(None if alpha is None else np.ascontiguousarray(alpha, dtype=np.float32)),
                                   1 if projection else 0, _lib.ptr(nd), _lib.ptr(na))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return nd, na


def remap_displacement(old_grid, new_grid, u, *, ctx=None):
    """Nodal displacements of old_grid interpolated onto new_grid (same box)
    as a warm start for the next solve (hexa_remap_displacement); float64."""
    ctx = ctx or context()
    nn = 3 * (new_grid.nx + 1) * (new_grid.ny + 1) * (new_grid.nz + 1)
    out = np.empty(nn, np.float64)
    rc = ctx.lib.hexa_remap_displacement(ctx.h, C.byref(old_grid), C.byref(new_grid),
                                         _lib.ptr(np.ascontiguousarray(u, dtype=np.float64)), _lib.ptr(out))
    ctx.check(rc, allow=(_lib.HEXA_OK,))
    return out


def refine_mesh_and_fields(grid, density, alpha, target_active, lengths, *, max_growth_rate=1.2,
                           hard_element_limit=800_000_000, update_method="hard", memory_limit=None, ctx=None):
    """Returns (grid, density, alpha, plan): the old ones when no refinement."""
    dens = np.asarray(density, dtype=np.float32)
    n_old = dens.size
    n_active = int(np.count_nonzero(dens > np.float32(0.001)))
    plan = plan_refinement(n_old, n_active, target_active, max_growth_rate=max_growth_rate,
                           hard_element_limit=hard_element_limit, memory_limit=memory_limit)
    if not plan.refine:
        return grid, density, alpha, plan
    nx, ny, nz, dx, dy, dz, count = element_distribution(*lengths, plan.new_total)
    ram = memory_limit if memory_limit is not None else hard_element_limit
    if count > ram:  # the post-distribution check of MeshRefiner.jl:151-155
        return grid, density, alpha, RefinePlan(False, n_old, "memory limit after distribution")
    new_grid = _lib.make_grid(nx, ny, nz, dx, dy, dz)
    nd, na = remap_fields(grid, new_grid, lengths, dens, alpha, projection=(update_method == "hard"), ctx=ctx)
    return new_grid, nd, na, plan
