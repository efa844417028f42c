"""On-disk formats either side of the SIMP loop: the "HEXA" v2 binary
file of the web viewer and the VTK XML ImageData (.vti) result file.

Restated from the reference's writers (host code, no GPU):
* ``export_binary_for_web`` (src/IO/Postprocessing.jl:370-471): little-endian
  header (UInt32 0x48455841, UInt32 version 2, Int32 iteration, Float32
  radius, Float32 threshold, UInt32 count, Float32 dx, dy, dz), then the
  Float32 centroids (3 per cell), densities and signed L1 stresses of the
  exported cells, then UInt32 length + JSON metadata.  Cells with
  density >= threshold are exported, thinned to ``max_export_cells`` by the
  reference's fractional stride; a cell's centroid is the Float32 mean of its
  8 node coordinates (MeshUtilities.jl:16-31) and its signed L1 carries the
  sign of the principal stress of largest magnitude (first wins ties).
* ``load_checkpoint`` (src/IO/Configuration.jl:32-78) reads the same file
  back; ``checkpoint_density`` rebuilds the full element field from the
  stored centroids (the reference's restart needs an unthinned file).
* ``export_solution_vti`` (src/IO/ExportVTK.jl:16-110): ImageData with
  appended raw Float32 cell arrays Density, L1_Stress, VonMises and, when the
  config asks for principal vectors, PrincipalValues, MaxPrincipalDirection,
  MinPrincipalDirection (3 components each), each prefixed by its UInt32 byte
  count.

The JSON metadata holds the same keys and values as the reference's; Julia's
``Dict`` has no defined key order, so the byte order of the keys may differ.
"""
from __future__ import annotations

import copy
import json
import struct

import numpy as np

HEXA_MAGIC = 0x48455841
HEXA_VERSION = 2
_HEADER = struct.Struct("<IIiffIfff")


def _f32(v) -> np.float32:
    return np.float32(v)


def export_indices(density, threshold, max_export_cells=0) -> np.ndarray:
    """0-based indices of the exported cells (Postprocessing.jl:384-402)."""
    dens = np.asarray(density, dtype=np.float32)
    active = np.nonzero(dens >= _f32(threshold))[0]
    n = active.size
    if max_export_cells > 0 and n > max_export_cells:
        step = n / max_export_cells
        picks = []
        cur = 1.0
        while cur <= n:
            picks.append(active[int(np.floor(cur)) - 1])
            cur += step
        return np.asarray(picks, dtype=np.int64)
    return active


def element_centroids(nx, ny, nz, dx, dy, dz, idx) -> np.ndarray:
    """Float32 centroids of cells idx (0-based, x fastest) as the mean of their
    8 node coordinates, summed in the node order n1..n8 of Mesh.jl:45-53."""
    idx = np.asarray(idx, dtype=np.int64)
    i = idx % nx
    j = (idx // nx) % ny
    k = idx // (nx * ny)
    di, dj, dk = (0, 1, 1, 0, 0, 1, 1, 0), (0, 0, 1, 1, 0, 0, 1, 1), (0, 0, 0, 0, 1, 1, 1, 1)
    out = np.zeros((idx.size, 3), dtype=np.float32)
    h = (_f32(dx), _f32(dy), _f32(dz))
    for a in range(8):
        for c, (ii, d) in enumerate(((i + di[a], h[0]), (j + dj[a], h[1]), (k + dk[a], h[2]))):
            out[:, c] += ii.astype(np.float32) * d
    return out * _f32(0.125)


def signed_l1(l1, principal) -> np.ndarray:
    """L1 stress with the sign of the principal stress of largest magnitude."""
    p = np.asarray(principal, dtype=np.float32).reshape(-1, 3)
    a = np.abs(p)
    sign = np.sign(p[:, 0])
    best = a[:, 0].copy()
    for c in (1, 2):
        take = a[:, c] > best
        best = np.where(take, a[:, c], best)
        sign = np.where(take, np.sign(p[:, c]), sign)
    return (np.asarray(l1, dtype=np.float32) * sign.astype(np.float32)).astype(np.float32)


def hexa_metadata(config: dict, iteration: int, radius: float, threshold: float) -> dict:
    """The JSON metadata of the binary file (Postprocessing.jl:406-424)."""
    meta = copy.deepcopy(config)
    meta["iteration"] = int(iteration)
    meta["radius"] = float(_f32(radius))
    meta["threshold"] = float(_f32(threshold))
    geom = meta.get("geometry")
    if isinstance(geom, dict):
        for shape in geom.values():
            if isinstance(shape, dict) and "type" in shape and "action" not in shape and "stiffness_ratio" in shape:
                shape["action"] = "add" if float(shape["stiffness_ratio"]) > 0 else "remove"
    meta["loads"] = config.get("external_forces", [])
    meta["bcs"] = config.get("boundary_conditions", [])
    meta["settings"] = config.get("optimization_parameters", {})
    return meta


def write_hexa_binary(path, grid, density, l1, principal, *, iteration, radius, threshold, config=None,
                      max_export_cells=0) -> int:
    """Write the v2 web file; returns the number of cells written (0: no file,
    as the reference writes nothing when no cell passes the threshold)."""
    idx = export_indices(density, threshold, max_export_cells)
    if idx.size == 0:
        return 0
    cent = element_centroids(grid.nx, grid.ny, grid.nz, grid.dx, grid.dy, grid.dz, idx)
    dens = np.asarray(density, dtype=np.float32)[idx]
    sl1 = signed_l1(np.asarray(l1, dtype=np.float32)[idx], np.asarray(principal, dtype=np.float32).reshape(-1, 3)[idx])
    blob = json.dumps(hexa_metadata(config or {}, iteration, radius, threshold)).encode("utf-8")
    with open(path, "wb") as fh:
        fh.write(_HEADER.pack(HEXA_MAGIC, HEXA_VERSION, int(iteration), float(_f32(radius)), float(_f32(threshold)),
                              int(idx.size), float(_f32(grid.dx)), float(_f32(grid.dy)), float(_f32(grid.dz))))
        fh.write(np.ascontiguousarray(cent, dtype="<f4").tobytes())
        fh.write(np.ascontiguousarray(dens, dtype="<f4").tobytes())
        fh.write(np.ascontiguousarray(sl1, dtype="<f4").tobytes())
        fh.write(struct.pack("<I", len(blob)))
        fh.write(blob)
    return int(idx.size)


def read_hexa_binary(path) -> dict:
    """Parse a v2 web file into its fields."""
    with open(path, "rb") as fh:
        data = fh.read()
    magic, version, iteration, radius, threshold, count, dx, dy, dz = _HEADER.unpack_from(data, 0)
    if magic != HEXA_MAGIC or version != HEXA_VERSION:
        raise ValueError(f"not a HEXA v2 file (magic {magic:#x}, version {version})")
    off = _HEADER.size
    cent = np.frombuffer(data, "<f4", 3 * count, off).reshape(count, 3)
    off += 12 * count
    dens = np.frombuffer(data, "<f4", count, off)
    off += 4 * count
    sl1 = np.frombuffer(data, "<f4", count, off)
    off += 4 * count
    (jlen,) = struct.unpack_from("<I", data, off)
    off += 4
    meta = json.loads(data[off:off + jlen].decode("utf-8"))
    if off + jlen != len(data):
        raise ValueError("trailing bytes after the JSON metadata")
    return dict(iteration=iteration, radius=radius, threshold=threshold, count=count, spacing=(dx, dy, dz),
                centroids=cent, density=dens, signed_l1=sl1, meta=meta)


def load_checkpoint(path):
    """Configuration.load_checkpoint (src/IO/Configuration.jl:32-78): returns
    (config, density, iteration, radius, threshold), density being the
    `count` stored values in file order."""
    d = read_hexa_binary(path)
    return d["meta"], np.array(d["density"], dtype=np.float32), int(d["iteration"]), np.float32(d["radius"]), \
        np.float32(d["threshold"])


def checkpoint_density(path, nx, ny, nz, dx, dy, dz, fill=1.0e-3) -> np.ndarray:
    """The full element field behind a checkpoint: each stored cell goes back
    to the element its centroid lies in (floor(c / d) per axis), every other
    element gets `fill`.  The reference's restart needs the stored count to
    equal the element count (Main.jl:269-271), which a file thresholded and
    thinned by export_binary_for_web (Postprocessing.jl:383-402) does not
    meet; this gives a full field either way."""
    d = read_hexa_binary(path)
    cent = np.asarray(d["centroids"], dtype=np.float64)
    h = np.array([dx, dy, dz], dtype=np.float64)
    ijk = np.floor(cent / h).astype(np.int64)
    n = np.array([nx, ny, nz])
    if ijk.size and (ijk.min() < 0 or np.any(ijk.max(axis=0) >= n)):
        raise ValueError("checkpoint cells lie outside the given grid")
    out = np.full(nx * ny * nz, np.float32(fill), dtype=np.float32)
    out[ijk[:, 0] + nx * (ijk[:, 1] + ny * ijk[:, 2])] = d["density"]
    return out


def _jl(v) -> str:
    """A Float32 as Julia's string() prints it (shortest round-trip form)."""
    s = np.format_float_positional(np.float32(v), unique=True, trim="0")
    return s if "." in s or "e" in s else s + ".0"


def write_vti(path, dims, spacing, origin, density, l1, vonmises, principal=None, dir_max=None, dir_min=None,
              config=None) -> str:
    """Write the .vti result file; the principal arrays are written when the
    config's output_settings.save_principal_stress_vectors is "yes"/true."""
    path = str(path)
    if not path.endswith(".vti"):
        path += ".vti"
    nx, ny, nz = dims
    n = int(np.asarray(density).size)
    sv = ((config or {}).get("output_settings", {}) or {}).get("save_principal_stress_vectors", "no")
    vectors = str(sv).lower() == "yes" or sv is True
    arrays = [("Density", density, 1), ("L1_Stress", l1, 1), ("VonMises", vonmises, 1)]
    if vectors:
        arrays += [("PrincipalValues", principal, 3), ("MaxPrincipalDirection", dir_max, 3),
                   ("MinPrincipalDirection", dir_min, 3)]
    extent = f"0 {nx} 0 {ny} 0 {nz}"
    head = ['<?xml version="1.0"?>\n', '<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">\n',
            f'  <ImageData WholeExtent="{extent}" Origin="{_jl(origin[0])} {_jl(origin[1])} {_jl(origin[2])}" '
            f'Spacing="{_jl(spacing[0])} {_jl(spacing[1])} {_jl(spacing[2])}">\n',
            f'    <Piece Extent="{extent}">\n',
            '      <CellData Scalars="Density" Vectors="MaxPrincipalDirection">\n']
    offset = 0
    for name, _, ncomp in arrays:
        comps = f' NumberOfComponents="{ncomp}"' if ncomp > 1 else ""
        head.append(f'        <DataArray type="Float32" Name="{name}"{comps} format="appended" offset="{offset}"/>\n')
        offset += 4 + 4 * n * ncomp
    head += ["      </CellData>\n", "    </Piece>\n", "  </ImageData>\n", '  <AppendedData encoding="raw">\n', "_"]
    with open(path, "wb") as fh:
        fh.write("".join(head).encode("ascii"))
        for _, arr, ncomp in arrays:
            a = np.ascontiguousarray(np.asarray(arr, dtype="<f4").reshape(-1))
            if a.size != n * ncomp:
                raise ValueError("array length does not match the cell count")
            fh.write(struct.pack("<I", a.nbytes))
            fh.write(a.tobytes())
        fh.write(b"\n  </AppendedData>\n</VTKFile>\n")
    return path


def read_vti_arrays(path) -> dict:
    """The appended Float32 cell arrays of a .vti written by write_vti."""
    import re
    data = open(path, "rb").read()
    tag = b'<AppendedData encoding="raw">\n_'
    start = data.index(tag) + len(tag)
    header = data[:start].decode("ascii")
    out = {}
    for m in re.finditer(r'Name="([^"]+)"(?: NumberOfComponents="(\d+)")? format="appended" offset="(\d+)"', header):
        name, ncomp, off = m.group(1), int(m.group(2) or 1), int(m.group(3))
        (nbytes,) = struct.unpack_from("<I", data, start + off)
        arr = np.frombuffer(data, "<f4", nbytes // 4, start + off + 4)
        out[name] = arr.reshape(-1, ncomp) if ncomp > 1 else arr
    return out
