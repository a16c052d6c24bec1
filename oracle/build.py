"""Build recipe of the CPU oracle (test infrastructure; see gales_oracle.cpp,
solver_oracle.cpp and magma_oracle.cpp) and of the reference's own classes that compile
here (ref_classes.cpp, from a checkout of the reference when one is present).

Compiled without floating-point contraction so that x86_64 and aarch64 hosts
give bit-identical results.  Output: oracle/_build/libgales_oracle.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRCS = [HERE / "gales_oracle.cpp", HERE / "solver_oracle.cpp", HERE / "magma_oracle.cpp"]
OUT = HERE / "_build" / "libgales_oracle.so"
# The reference's own classes that compile here (ref_classes.cpp), built from a checkout
# of the reference where one is present; output only into oracle/_ref/.
REF_DIR = Path(os.environ.get("GALES_REFERENCE_DIR", "/root/reference"))
REF_SRC = HERE / "ref_classes.cpp"
REF_OUT = HERE / "_ref" / "libref_classes.so"


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


def build_ref(verbose: bool = False):
    """Compile ref_classes.cpp against the reference's headers where they lie in the
    checkout (fluid/chemicals.hpp, base_chemical.hpp, GiordanoEtAlViscosityModel.hpp;
    mesh/element.hpp, node.hpp, point.hpp).  Returns the library path, or None without
    a checkout."""
    inc = REF_DIR / "src" / "fem" / "physical_props" / "fluid"
    mesh = REF_DIR / "src" / "fem" / "mesh"
    if not (inc / "chemicals.hpp").exists() or not (mesh / "element.hpp").exists():
        return None
    REF_OUT.parent.mkdir(exist_ok=True)
    deps = [REF_SRC, inc / "chemicals.hpp", inc / "base_chemical.hpp", inc / "GiordanoEtAlViscosityModel.hpp",
            mesh / "element.hpp", mesh / "node.hpp", mesh / "point.hpp"]
    if REF_OUT.exists() and REF_OUT.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return REF_OUT
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(inc), "-I", str(mesh),
           "-o", str(REF_OUT), str(REF_SRC)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("building the reference's property classes failed")
    return REF_OUT


if __name__ == "__main__":
    print(build(verbose=True))
    print(build_ref(verbose=True))
