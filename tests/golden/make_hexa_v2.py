"""Builds tests/golden/hexa_v2_fixture.json: the bytes the reference's HEXA v2
web writer puts before its JSON metadata, for one small hand-chosen case.

The bytes are derived here step by step from the reference's own code, with
no use of the package under test:
  * Mesh.jl:36-39 / 44-53 — node coordinates (i-1)*dx in Float32 (x fastest)
    and the element node order n1..n8;
  * MeshUtilities.jl:16-30 — element_centroid: Float32 sums over n1..n8,
    then times 0.125f0;
  * Postprocessing.jl:383-401 — active cells (density >= threshold) and the
    fractional-stride subsample when max_export_cells is exceeded;
  * Postprocessing.jl:430-464 — header (UInt32 magic 0x48455841, UInt32 2,
    Int32 iter, Float32 radius, Float32 threshold, UInt32 count, Float32
    dx/dy/dz), then centroids, densities and signed L1 (first principal of
    largest |.| by strict '>', sign(0) = 0) as little-endian Float32 arrays.
The JSON that follows (JSON.json of a Julia Dict, whose key order is the
Dict's hash order) is not byte-pinned; the test compares its content.

Run: python tests/golden/make_hexa_v2.py
"""
import json
import math
import pathlib
import struct

import numpy as np

F = np.float32
NX, NY, NZ = 3, 2, 2
DX, DY, DZ = 0.3, 0.7, 1.1  # not dyadic: the Float32 summation order shows in the bits
ITER, RADIUS, THRESHOLD, MAX_CELLS = 12, 1.75, 0.3, 7

DENSITY = [0.05, 0.3, 0.31, 0.9, 0.299, 1.0, 0.5, 0.3, 0.75, 0.2, 0.6, 0.45]
L1 = [1.5, 2.25, 0.0, 3.0, 4.5, 1.0, 2.0, 6.5, 0.75, 1.25, 9.0, 0.5]
PRINCIPAL = [[1.0, -2.0, 0.5], [-3.0, 3.0, 1.0], [0.0, 0.0, 0.0], [2.0, -2.5, 2.5],
             [0.25, 0.5, -0.75], [-1.0, 0.0, 0.0], [4.0, -4.0, -4.0], [0.0, -0.0, 1e-3],
             [-0.5, 0.25, 0.125], [1.0, 1.0, -1.0], [-7.0, 6.0, 7.0], [0.0, 2.0, -1.0]]


def julia_sign(v):
    return F(0.0) if v == 0 else F(math.copysign(1.0, float(v)))


def main():
    dx, dy, dz = F(DX), F(DY), F(DZ)
    nnx, nny, nnz = NX + 1, NY + 1, NZ + 1
    nodes = []  # Mesh.jl:36-39, 1-based i, j, k
    for k in range(1, nnz + 1):
        for j in range(1, nny + 1):
            for i in range(1, nnx + 1):
                nodes.append((F(i - 1) * dx, F(j - 1) * dy, F(k - 1) * dz))

    def node_index(i, j, k):
        return i + (j - 1) * nnx + (k - 1) * nnx * nny

    elements = []  # Mesh.jl:44-53
    for k in range(1, NZ + 1):
        for j in range(1, NY + 1):
            for i in range(1, NX + 1):
                elements.append([node_index(i, j, k), node_index(i + 1, j, k), node_index(i + 1, j + 1, k),
                                 node_index(i, j + 1, k), node_index(i, j, k + 1), node_index(i + 1, j, k + 1),
                                 node_index(i + 1, j + 1, k + 1), node_index(i, j + 1, k + 1)])

    density = [F(v) for v in DENSITY]
    thr = F(THRESHOLD)
    active = [e for e in range(1, len(density) + 1) if density[e - 1] >= thr]  # 1-based, findall
    n_active = len(active)
    if MAX_CELLS > 0 and n_active > MAX_CELLS:  # Postprocessing.jl:387-398 (Float64 stride)
        step = n_active / MAX_CELLS
        chosen, cur = [], 1.0
        while cur <= n_active:
            ii = math.floor(cur)
            if ii <= n_active:
                chosen.append(active[ii - 1])
            cur += step
    else:
        chosen = active
    count = len(chosen)

    out = bytearray()
    out += struct.pack("<I", 0x48455841) + struct.pack("<I", 2) + struct.pack("<i", ITER)
    out += struct.pack("<f", F(RADIUS)) + struct.pack("<f", thr) + struct.pack("<I", count)
    out += struct.pack("<f", dx) + struct.pack("<f", dy) + struct.pack("<f", dz)
    cent, dens, sl1 = [], [], []
    inv8 = F(0.125)
    for e in chosen:  # MeshUtilities.element_centroid, Postprocessing.jl:445-459
        cx = cy = cz = F(0.0)
        for n in elements[e - 1]:
            x, y, z = nodes[n - 1]
            cx = F(cx + x)
            cy = F(cy + y)
            cz = F(cz + z)
        cent += [F(cx * inv8), F(cy * inv8), F(cz * inv8)]
        dens.append(density[e - 1])
        s = [F(v) for v in PRINCIPAL[e - 1]]
        abs_max, sgn = abs(s[0]), julia_sign(s[0])
        if abs(s[1]) > abs_max:
            abs_max, sgn = abs(s[1]), julia_sign(s[1])
        if abs(s[2]) > abs_max:
            abs_max, sgn = abs(s[2]), julia_sign(s[2])
        sl1.append(F(F(L1[e - 1]) * sgn))
    for v in cent + dens + sl1:
        out += struct.pack("<f", v)
    fixture = {"grid": [NX, NY, NZ], "spacing": [DX, DY, DZ], "iteration": ITER, "radius": RADIUS,
               "threshold": THRESHOLD, "max_export_cells": MAX_CELLS, "density": DENSITY, "l1": L1,
               "principal": PRINCIPAL, "count": count, "cells_1based": chosen, "prefix_hex": out.hex()}
    path = pathlib.Path(__file__).with_name("hexa_v2_fixture.json")
    path.write_text(json.dumps(fixture, indent=1) + "\n")
    print(f"wrote {path} ({count} cells, {len(out)} bytes before the JSON length)")


if __name__ == "__main__":
    main()
