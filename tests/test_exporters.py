"""The on-disk formats either side of the loop (host code): the HEXA v2 web
binary (Postprocessing.jl:370-471) and the .vti result file
(ExportVTK.jl:16-110), written and parsed back byte by byte."""
import struct

import numpy as np

from v119_2025_12_19_hexatop_aws_gb300 import _lib
from v119_2025_12_19_hexatop_aws_gb300.exporters import (checkpoint_density, export_indices, load_checkpoint,
                                                         read_hexa_binary, read_vti_arrays, signed_l1,
                                                         write_hexa_binary, write_vti)


def test_export_indices_threshold_and_fractional_stride():
    dens = np.array([0.1, 0.6, 0.7, 0.2, 0.9, 0.95, 0.5, 0.8, 0.99, 0.51, 0.52, 0.3], dtype=np.float32)
    act = np.nonzero(dens >= 0.5)[0]  # 9 cells
    assert np.array_equal(export_indices(dens, 0.5), act)
    # 9 active, at most 4: stride 2.25 -> 1-based picks 1, 3.25, 5.5, 7.75 -> floor 1, 3, 5, 7
    assert np.array_equal(export_indices(dens, 0.5, 4), act[[0, 2, 4, 6]])


def test_signed_l1_takes_the_sign_of_the_largest_principal():
    p = np.array([[3.0, 1.0, -5.0], [4.0, 0.0, -4.0], [-1.0, -2.0, -0.5]], dtype=np.float32)
    l1 = np.abs(p).sum(axis=1).astype(np.float32)
    assert np.array_equal(signed_l1(l1, p), np.array([-9.0, 8.0, -3.5], dtype=np.float32))


def test_hexa_binary_layout_and_round_trip(tmp_path):
    grid = _lib.make_grid(4, 3, 2, 1.0, 2.0, 0.5)
    ne = 24
    rng = np.random.default_rng(3)
    dens = rng.uniform(0, 1, ne).astype(np.float32)
    principal = rng.standard_normal((ne, 3)).astype(np.float32)
    l1 = np.abs(principal).sum(axis=1).astype(np.float32)
    cfg = {"geometry": {"hole": {"type": "sphere", "stiffness_ratio": 0.0}}, "external_forces": [{"F": [0, 0, -1]}],
           "boundary_conditions": [{"location": [0, ":", ":"]}], "optimization_parameters": {"volfrac": 0.3}}
    path = tmp_path / "iter.bin"
    n = write_hexa_binary(path, grid, dens, l1, principal, iteration=7, radius=1.5, threshold=0.3, config=cfg)
    idx = np.nonzero(dens >= 0.3)[0]
    assert n == idx.size
    raw = path.read_bytes()
    magic, ver, it, rad, thr, cnt, dx, dy, dz = struct.unpack_from("<IIiffIfff", raw, 0)
    assert (magic, ver, it, cnt) == (0x48455841, 2, 7, idx.size)
    assert raw[:4] == b"AXEH"  # the UInt32 magic as a little-endian file writes it
    assert (rad, thr, dx, dy, dz) == (1.5, np.float32(0.3), 1.0, 2.0, 0.5)
    back = read_hexa_binary(path)
    i, j, k = idx % 4, (idx // 4) % 3, idx // 12
    assert np.allclose(back["centroids"], np.stack([(i + 0.5) * 1.0, (j + 0.5) * 2.0, (k + 0.5) * 0.5], 1), atol=1e-6)
    assert np.array_equal(back["density"], dens[idx])
    assert np.array_equal(back["signed_l1"], signed_l1(l1[idx], principal[idx]))
    meta = back["meta"]
    assert meta["iteration"] == 7 and meta["loads"] == cfg["external_forces"] and meta["bcs"] == cfg["boundary_conditions"]
    assert meta["settings"] == {"volfrac": 0.3} and meta["geometry"]["hole"]["action"] == "remove"
    assert len(raw) == 36 + 20 * idx.size + 4 + struct.unpack_from("<I", raw, 36 + 20 * idx.size)[0]


def test_hexa_binary_matches_the_reference_writer_bytes(tmp_path):
    """Every byte before the JSON metadata equals the bytes derived step by
    step from the reference writer (tests/golden/make_hexa_v2.py: non-dyadic
    spacing, threshold ties, the fractional-stride subsample, sign ties and
    zeros); the JSON is compared by content (its key order is a Julia Dict's)."""
    import json
    import pathlib
    fx = json.loads((pathlib.Path(__file__).parent / "golden" / "hexa_v2_fixture.json").read_text())
    grid = _lib.make_grid(*fx["grid"], *fx["spacing"])
    cfg = {"external_forces": [{"F": [0, 0, -1]}], "optimization_parameters": {"volfrac": 0.3}}
    path = tmp_path / "golden.bin"
    n = write_hexa_binary(path, grid, np.array(fx["density"], np.float32), np.array(fx["l1"], np.float32),
                          np.array(fx["principal"], np.float32), iteration=fx["iteration"], radius=fx["radius"],
                          threshold=fx["threshold"], config=cfg, max_export_cells=fx["max_export_cells"])
    assert n == fx["count"]
    raw = path.read_bytes()
    prefix = bytes.fromhex(fx["prefix_hex"])
    assert raw[:len(prefix)] == prefix
    (jlen,) = struct.unpack_from("<I", raw, len(prefix))
    meta = json.loads(raw[len(prefix) + 4:].decode("utf-8"))
    assert len(raw) == len(prefix) + 4 + jlen
    assert meta["iteration"] == fx["iteration"] and meta["loads"] == cfg["external_forces"]
    assert meta["bcs"] == [] and meta["settings"] == {"volfrac": 0.3}
    assert np.float32(meta["radius"]) == np.float32(fx["radius"])
    assert np.float32(meta["threshold"]) == np.float32(fx["threshold"])


def test_hexa_binary_writes_nothing_without_active_cells(tmp_path):
    grid = _lib.make_grid(2, 2, 2)
    path = tmp_path / "none.bin"
    n = write_hexa_binary(path, grid, np.zeros(8, np.float32), np.zeros(8, np.float32), np.zeros((8, 3), np.float32),
                          iteration=1, radius=1.0, threshold=0.5)
    assert n == 0 and not path.exists()


def test_vti_header_and_arrays(tmp_path):
    rng = np.random.default_rng(4)
    dims = (3, 2, 2)
    n = 12
    dens, l1, vm = (rng.uniform(0, 1, n).astype(np.float32) for _ in range(3))
    pv, dmax, dmin = (rng.standard_normal((n, 3)).astype(np.float32) for _ in range(3))
    for vectors in ("no", "yes"):
        path = write_vti(tmp_path / f"res_{vectors}", dims, (1.0, 2.0, 0.5), (0.0, 0.0, 0.0), dens, l1, vm, pv, dmax,
                         dmin, config={"output_settings": {"save_principal_stress_vectors": vectors}})
        text = open(path, "rb").read().split(b"<AppendedData")[0].decode()
        assert '<ImageData WholeExtent="0 3 0 2 0 2" Origin="0.0 0.0 0.0" Spacing="1.0 2.0 0.5">' in text
        assert 'Name="L1_Stress" format="appended" offset="52"' in text  # 4 + 12 * 4 after Density
        arrs = read_vti_arrays(path)
        assert np.array_equal(arrs["Density"], dens) and np.array_equal(arrs["VonMises"], vm)
        if vectors == "yes":
            assert np.array_equal(arrs["PrincipalValues"], pv) and np.array_equal(arrs["MinPrincipalDirection"], dmin)
        else:
            assert "PrincipalValues" not in arrs
        assert open(path, "rb").read().endswith(b"\n  </AppendedData>\n</VTKFile>\n")


def test_checkpoint_reload_and_full_field(tmp_path):
    """load_checkpoint returns what Configuration.load_checkpoint returns; the
    full field is rebuilt from the stored centroids even from a thresholded,
    thinned file (the reference's restart needs count == nElem)."""
    dims, h = (10, 6, 4), (0.5, 1.0, 2.0)
    grid = _lib.make_grid(*dims, *h)
    ne = 240
    rng = np.random.default_rng(8)
    dens = rng.uniform(0, 1, ne).astype(np.float32)
    princ = rng.standard_normal((ne, 3)).astype(np.float32)
    l1 = np.abs(princ).sum(axis=1).astype(np.float32)
    cfg = {"number_of_iterations": 30, "optimization_parameters": {"min_density": 0.001}}
    path = tmp_path / "ck.bin"
    n = write_hexa_binary(path, grid, dens, l1, princ, iteration=12, radius=0.75, threshold=0.3, config=cfg,
                          max_export_cells=50)
    config, d, it, r, thr = load_checkpoint(path)
    assert n == 50 and d.size == 50 and it == 12 and r == np.float32(0.75) and thr == np.float32(0.3)
    assert config["number_of_iterations"] == 30 and config["iteration"] == 12
    idx = export_indices(dens, 0.3, 50)
    assert np.array_equal(d, dens[idx])
    full = checkpoint_density(path, *dims, *h, fill=0.001)
    expect = np.full(ne, np.float32(0.001))
    expect[idx] = dens[idx]
    assert np.array_equal(full, expect)
    # every cell stored: the original field comes back exactly
    write_hexa_binary(path, grid, dens, l1, princ, iteration=1, radius=0.5, threshold=0.0, config=cfg)
    assert np.array_equal(checkpoint_density(path, *dims, *h), dens)

