"""The C-ABI library loads, exports every symbol include/hexagpu.h declares,
and its host-only entry points (element matrices, defaults) agree with the
oracle.  No compute call here needs a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from v119_2025_12_19_hexatop_aws_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "hexagpu.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(hexa_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_symbols():
    assert declared_functions() == sorted(_lib.SIGNATURES)


def test_header_cites_the_reference_for_every_entry_point():
    """Each declaration's comment block (or its section's) names the
    reference file it replaces, or says that the reference has no counterpart."""
    text = HEADER.read_text()
    missing = []
    last_comment = ""
    for m in re.finditer(r"(/\*.*?\*/)|\b(?:int|void|double|int64_t|const char\*)\s+(hexa_[a-z0-9_]+)\s*\(", text, re.S):
        if m.group(1):
            last_comment = m.group(1) if ".jl" in m.group(1) or "counterpart" in m.group(1) else last_comment
            continue
        if ".jl" not in last_comment and "counterpart" not in last_comment:
            missing.append(m.group(2))
    assert missing == []


def test_integration_guide_covers_every_entry_point():
    doc = (HEADER.parents[1] / "INTEGRATION.md").read_text()
    assert [n for n in declared_functions() if f"`{n}`" not in doc] == []


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing


def test_bound_loader(built_lib):
    lib = _lib.load()
    assert lib.hexa_version() >= 100


def test_host_stiffness_matches_oracle(built_lib, oracle):
    for dims, nu in [((1, 1, 1), 0.3), ((1, 2, 0.5), 0.3), ((0.3, 1.7, 2.9), 0.45)]:
        k = np.empty(576)
        assert _lib.load().hexa_canonical_stiffness(*dims, nu, _lib.ptr(k)) == 0
        K = k.reshape(24, 24, order="F")
        Ko = oracle.canonical_stiffness(*dims, nu)
        assert np.abs(K - Ko).max() <= 1e-15 * np.abs(Ko).max() * 8


def test_host_stiffness_rejects_bad_geometry(built_lib):
    k = np.empty(576)
    assert _lib.load().hexa_canonical_stiffness(0.0, 1, 1, 0.3, _lib.ptr(k)) != 0
    assert _lib.load().hexa_canonical_stiffness(1, 1, 1, 0.5, _lib.ptr(k)) != 0


@pytest.mark.parametrize("quirk", [0, 1])
def test_host_scalar_matrices_match_oracle(built_lib, oracle, quirk):
    ke, me = np.empty(64), np.empty(64)
    assert _lib.load().hexa_scalar_canonical_matrices(1.0, 2.0, 0.5, quirk, _lib.ptr(ke), _lib.ptr(me)) == 0
    Ke, Me = oracle.scalar_matrices(1.0, 2.0, 0.5, bool(quirk))
    assert np.allclose(ke.reshape(8, 8, order="F"), Ke, rtol=0, atol=1e-15)
    assert np.allclose(me.reshape(8, 8, order="F"), Me, rtol=0, atol=1e-15)


def test_default_params(built_lib):
    p = _lib.default_params()
    assert p.tol == 1e-9 and p.precond == 1 and p.shift_factor == 1e-10 and p.diag_quirk == 1
    q = _lib.default_params(precision="mixed", precond="jacobi", mg_levels=4)
    assert q.precision == 1 and q.precond == 0 and q.mg_levels == 4
    with pytest.raises(KeyError):
        _lib.default_params(not_a_key=1)


def test_default_density_update_params(built_lib):
    p = _lib.DensityUpdateParams()
    _lib.load(built_lib).hexa_default_density_update_params(C.byref(p))
    assert p.min_density == np.float32(1e-3) and p.max_density == 1.0 and p.filter_R_interm_iter_perc == 50.0
    assert p.minimum_filter_radius_as_elements == 2.5 and p.filter_tolerance == np.float32(1e-5)
    assert p.final_density_threshold == np.float32(0.95) and p.max_culling_ratio == np.float32(0.1)
    assert p.hard_update == 0 and p.filter_max_iter == 200 and p.filter_precision == 2


def test_struct_sizes_match_header_layout(built_lib):
    # 8-byte aligned doubles after int32 pairs: sizes computed by the C compiler
    assert C.sizeof(_lib.Grid) == 40
    assert C.sizeof(_lib.BC) == 16
    assert C.sizeof(_lib.SolveParams) % 8 == 0


def test_ctypes_layout_matches_c_compiler(tmp_path):
    """offsetof/sizeof of every public struct, from gcc on include/hexagpu.h."""
    import subprocess
    structs = {"hexa_grid": _lib.Grid, "hexa_bc": _lib.BC, "hexa_solve_params": _lib.SolveParams,
               "hexa_solve_stats": _lib.SolveStats, "hexa_filter_stats": _lib.FilterStats,
               "hexa_density_update_params": _lib.DensityUpdateParams,
               "hexa_density_update_stats": _lib.DensityUpdateStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n") if l)
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(py, f).offset, f"{cname}.{f}"
