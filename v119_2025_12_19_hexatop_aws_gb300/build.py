"""In-tree build of libhexagpu.so for sm_103a (GB300).

Each translation unit under csrc/ is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``libhexagpu.so`` next to this file.  No cmake, no torch extension machinery:
the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhexagpu.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["op.cu", "vec.cu", "mg.cu", "helm.cu", "topo.cu", "block.cu", "batch.cu", "stress.cu", "remap.cu", "update.cu", "solver.cu", "capi.cu", "noalloc.cu", "element.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhexagpu.so")


def _flags(src: str, ptxas_verbose: bool) -> list[str]:
    # host code without FMA contraction: the same roundings on x86-64 and aarch64
    f = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-lineinfo",
         "--expt-relaxed-constexpr"]
    if src.endswith(".cu"):
        f += [ARCH]
        if ptxas_verbose:
            f += ["-Xptxas", "-v"]
    else:
        f += ["-x", "cu", ARCH]  # host-only C++ compiled by nvcc so one toolchain links everything
    return f


def _compile(src: str, ptxas_verbose: bool) -> tuple[str, str]:
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), "-c", str(CSRC / src), "-o", str(obj), f"-I{CSRC}", f"-I{PKG.parent / 'include'}"]
    cmd += _flags(src, ptxas_verbose)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return str(obj), r.stderr


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "hexagpu.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compile and link libhexagpu.so if any source is newer than it."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    jobs = min(len(SOURCES), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), SOURCES))
    if verbose or ptxas_verbose:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp), *[o for o, _ in results], ARCH, "-cudart", "static", "-lrt", "-lpthread", "-ldl",
           "-Xlinker", "--no-undefined"]  # a missing definition fails the build, not the first call
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
