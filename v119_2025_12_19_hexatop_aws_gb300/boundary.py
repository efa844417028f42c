"""Boundary-condition and load input semantics (src/Core/Boundary.jl).

Host-side only: these build the ``bc_indicator`` and ``F`` arrays the solve
entry point takes, with the reference's location grammar
(Boundary.jl:52-130): ``":"`` matches all, a number in [0,1] is a FRACTION of
the extent (Boundary.jl:119), other numbers are coordinates, ``"NN%"`` is a
percentage; matching uses tol = 1e-4 * max(1, extent).  Forces given by
location are spread evenly over the matched nodes (Boundary.jl:280) and an
empty point match falls back to the nearest node (Boundary.jl:195-224,
250-265).
"""
from __future__ import annotations

import numpy as np


def _resolve(spec, cmin: np.float32, cmax: np.float32) -> np.float32:
    """resolve_coordinate_value (Boundary.jl:117-130)."""
    if isinstance(spec, str) and spec.endswith("%"):
        frac = np.float32(float(spec[:-1])) / np.float32(100.0)
        frac = np.clip(frac, np.float32(0.0), np.float32(1.0))
        return np.float32(cmin + frac * (cmax - cmin))
    if isinstance(spec, (int, float, np.number)) and not isinstance(spec, bool):
        if 0.0 <= spec <= 1.0:
            return np.float32(cmin + np.float32(spec) * (cmax - cmin))
        return np.float32(spec)
    return np.float32(cmin)


def _component_mask(spec, coords: np.ndarray) -> np.ndarray:
    """interpret_location_component (Boundary.jl:79-115)."""
    cmin, cmax = np.float32(coords.min()), np.float32(coords.max())
    tol = np.float32(1e-4) * max(np.float32(1.0), abs(cmax - cmin))
    if isinstance(spec, str) and spec == ":":
        return np.ones(coords.shape[0], dtype=bool)
    if (isinstance(spec, (int, float, np.number)) and not isinstance(spec, bool)) or (
            isinstance(spec, str) and spec.endswith("%")):
        val = _resolve(spec, cmin, cmax)
        return np.abs(coords - val) <= tol
    raise ValueError(f"Invalid location component: {spec!r}")


def nodes_by_location(loc, nodes: np.ndarray) -> np.ndarray:
    """0-based indices of nodes matching a location triple (Boundary.jl:52-77)."""
    if len(loc) < 3:
        raise ValueError("Location specification must have at least 3 components (x,y,z)")
    m = np.ones(nodes.shape[0], dtype=bool)
    for d in range(3):
        m &= _component_mask(loc[d], nodes[:, d].astype(np.float32))
    return np.nonzero(m)[0]


def affected_nodes(spec: dict, nodes: np.ndarray) -> np.ndarray:
    """get_affected_nodes (Boundary.jl:18-50); returns 0-based indices."""
    n = nodes.shape[0]
    if "node" in spec:
        raw = spec["node"]
        if isinstance(raw, (int, np.integer)):
            return np.array([int(np.clip(raw, 1, n)) - 1])
        return np.unique(np.clip(np.asarray(raw, dtype=np.int64), 1, n)) - 1
    if "location" in spec:
        return nodes_by_location(spec["location"], nodes)
    raise ValueError("Specification must include either 'node' or 'location'")


def get_bc_indicator(nNodes: int, nodes: np.ndarray, bc_data: list) -> np.ndarray:
    """(nNodes, 3) Float32, 1 where a DOF is fixed (Boundary.jl:135-160)."""
    bc = np.zeros((nNodes, 3), dtype=np.float32)
    for spec in bc_data:
        dofs = list(spec["DoFs"])
        for d in dofs:
            if d < 1 or d > 3:
                raise ValueError(f"Invalid DoF index: {d} (must be 1..3).")
        idx = affected_nodes(spec, nodes)
        for d in dofs:
            bc[idx, d - 1] = 1.0
    return bc


def _nearest_node(target: np.ndarray, nodes: np.ndarray) -> int:
    """find_nearest_node (Boundary.jl:195-224) with its tie-break on larger x, y, z."""
    best, best_d = -1, np.inf
    for i in range(nodes.shape[0]):
        d = float(np.sum((nodes[i] - target) ** 2))
        if d < best_d - 1e-9:
            best, best_d = i, d
        elif abs(d - best_d) <= 1e-9 and best >= 0:
            if tuple(nodes[i]) > tuple(nodes[best]):
                best = i
    return best


def apply_external_forces(F: np.ndarray, forces_data: list, nodes: np.ndarray) -> np.ndarray:
    """Adds loads to the interleaved xyz vector F in place (Boundary.jl:232-291)."""
    bounds = [(np.float32(nodes[:, d].min()), np.float32(nodes[:, d].max())) for d in range(3)]
    for force in forces_data:
        idx = affected_nodes(force, nodes)
        if idx.size == 0 and "location" in force:
            loc = force["location"]
            if all(not (isinstance(c, str) and c == ":") for c in loc):
                target = np.array([_resolve(loc[d], *bounds[d]) for d in range(3)], dtype=np.float32)
                nn = _nearest_node(target, nodes)
                if nn >= 0:
                    idx = np.array([nn])
        if idx.size == 0:
            continue
        f = np.zeros(3, dtype=F.dtype)
        raw = list(force["F"])[:3]
        f[:len(raw)] = raw
        scale = (1.0 / idx.size) if "location" in force else 1.0
        for c in range(3):
            np.add.at(F, 3 * idx + c, F.dtype.type(scale) * f[c])
    return F


def bc_to_fixed_dof(bc_indicator: np.ndarray) -> np.ndarray:
    """Per-DOF byte mask (nonzero = fixed) from the (nNodes,3) indicator (GPUSolver.jl:170-180)."""
    return np.ascontiguousarray((np.asarray(bc_indicator) > 0).astype(np.uint8).reshape(-1))


def face_clamps(fixed_dof: np.ndarray, nx: int, ny: int, nz: int):
    """Split a per-DOF mask into whole-face clamps (bit f: x-,x+,y-,y+,z-,z+) and
    the remainder; the remainder is None when the faces cover the mask."""
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    m = np.asarray(fixed_dof, dtype=bool).reshape(NZ, NY, NX, 3)
    faces, covered = 0, np.zeros_like(m)
    sel = [(0, np.s_[:, :, 0]), (1, np.s_[:, :, -1]), (2, np.s_[:, 0, :]), (3, np.s_[:, -1, :]),
           (4, np.s_[0, :, :]), (5, np.s_[-1, :, :])]
    for bit, s in sel:
        if m[s].all():
            faces |= 1 << bit
            covered[s] = True
    rest = m & ~covered
    return faces, (None if not rest.any() else np.ascontiguousarray(m.reshape(-1).astype(np.uint8)))
