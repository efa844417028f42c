"""Builds the oracle's C restatement (oracle/_build/libhexa_oracle.so).

TEST INFRASTRUCTURE: the oracle is the parity checker and the timed CPU
baseline; nothing in the product links it.  The reference itself is Julia
(CUDA.jl), which has no C sources to compile here, so there is no
oracle/_ref build: the restatement is the whole oracle.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "hexa_oracle.c"
OUT = HERE / "_build" / "libhexa_oracle.so"


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    tmp = OUT.with_suffix(".so.tmp")
    # no FMA contraction: Julia rounds each product and sum, and x86-64 and aarch64 then agree
    cmd = [cc, "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
