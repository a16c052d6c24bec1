"""Build recipe of the CPU oracle (test infrastructure; see gales_oracle.cpp,
solver_oracle.cpp and magma_oracle.cpp).

Compiled without floating-point contraction so that x86_64 and aarch64 hosts
give bit-identical results.  Output: oracle/_build/libgales_oracle.so.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRCS = [HERE / "gales_oracle.cpp", HERE / "solver_oracle.cpp", HERE / "magma_oracle.cpp"]
OUT = HERE / "_build" / "libgales_oracle.so"


def build(verbose: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    hdr = HERE.parent / "include" / "gales_asm.h"
    if OUT.exists() and OUT.stat().st_mtime > max([s.stat().st_mtime for s in SRCS] + [hdr.stat().st_mtime]):
        return OUT
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", str(OUT), *[str(s) for s in SRCS]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("building the oracle failed")
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
