"""The C ABI from a plain C program (tests/c_driver/abi_driver.c), linked
against the in-tree libhexagpu.so with gcc: host-only entry points here, a
small solve, filter and density update on the GPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _driver(built_lib, tmp_path):
    lib = Path(built_lib)
    exe = tmp_path / "abi_driver"
    subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", str(ROOT / "tests" / "c_driver" / "abi_driver.c"),
                    f"-I{ROOT / 'include'}", f"-L{lib.parent}", "-lhexagpu", f"-Wl,-rpath,{lib.parent}", "-lm",
                    "-o", str(exe)], check=True)
    return exe


def test_c_driver_host_entry_points(built_lib, tmp_path):
    r = subprocess.run([str(_driver(built_lib, tmp_path))], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok host"


@pytest.mark.gpu
def test_c_driver_on_the_gpu(built_lib, tmp_path):
    r = subprocess.run([str(_driver(built_lib, tmp_path)), "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok gpu"
