"""Structured hex8 mesh: the layout contract of src/Mesh/Mesh.jl:13-60.

Nodes are numbered x fastest, 1-based in the reference
(``node_index(i,j,k) = i + (j-1)*NX + (k-1)*NX*NY``); element node order
n1..n8 is (i,j,k), (i+1,j,k), (i+1,j+1,k), (i,j+1,k) and the same four at k+1
(Mesh.jl:44-53).  The GPU library only needs the grid dimensions, so a caller
passing ``nodes``/``elements`` arrays is checked against this generator, as
the Julia shim does before it calls into the library.
"""
from __future__ import annotations

import numpy as np


def node_index(i, j, k, nNodes_x, nNodes_y):
    """1-based node index of 1-based (i, j, k) (Mesh.jl:17-19)."""
    return i + (j - 1) * nNodes_x + (k - 1) * nNodes_x * nNodes_y


def generate_mesh(nx: int, ny: int, nz: int, dx: float = 1.0, dy: float = 1.0, dz: float = 1.0):
    """(nodes Float32 (nNodes,3), elements Int64 (nElem,8) 1-based, dims) as Mesh.generate_mesh."""
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    k, j, i = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    nodes = np.stack([(i * np.float32(dx)).ravel(), (j * np.float32(dy)).ravel(), (k * np.float32(dz)).ravel()],
                     axis=1).astype(np.float32)
    ek, ej, ei = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    n1 = (ei + NX * (ej + NY * ek)).ravel() + 1
    off = [0, 1, 1 + NX, NX, NX * NY, 1 + NX * NY, 1 + NX + NX * NY, NX + NX * NY]
    elements = np.stack([n1 + o for o in off], axis=1).astype(np.int64)
    return nodes, elements, (NX, NY, NZ)


def structured_dims(nodes: np.ndarray, elements: np.ndarray):
    """Recover (nx, ny, nz, dx, dy, dz) from a mesh that equals generate_mesh's.

    Raises ValueError for any other mesh (e.g. one pruned by MeshPruner),
    because the structured kernels cannot take it."""
    nodes = np.asarray(nodes)
    elements = np.asarray(elements)
    if nodes.ndim != 2 or nodes.shape[1] != 3 or elements.ndim != 2 or elements.shape[1] != 8:
        raise ValueError("nodes must be (nNodes,3) and elements (nElem,8)")
    x, y, z = (np.unique(nodes[:, d]) for d in range(3))
    NX, NY, NZ = len(x), len(y), len(z)
    if NX * NY * NZ != nodes.shape[0] or (NX - 1) * (NY - 1) * (NZ - 1) != elements.shape[0]:
        raise ValueError("mesh is not a full structured brick (pruned or unstructured meshes are not supported)")
    dx = float(x[1] - x[0]) if NX > 1 else 1.0
    dy = float(y[1] - y[0]) if NY > 1 else 1.0
    dz = float(z[1] - z[0]) if NZ > 1 else 1.0
    ref_nodes, ref_elems, _ = generate_mesh(NX - 1, NY - 1, NZ - 1, dx, dy, dz)
    if not np.array_equal(np.asarray(elements, dtype=np.int64), ref_elems):
        raise ValueError("element connectivity differs from the structured numbering of Mesh.jl")
    if not np.allclose(nodes - nodes[0], ref_nodes, rtol=0, atol=1e-4 * max(dx, dy, dz)):
        raise ValueError("node coordinates are not a uniform brick lattice")
    return NX - 1, NY - 1, NZ - 1, dx, dy, dz
