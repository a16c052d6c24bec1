"""Build the CUDA assembly library libgales_asm.so in-tree for sm_103a.

Each element type's kernels are a separate translation unit, compiled in
parallel; the host/C-ABI unit is linked with them into one shared library next
to this file.  Objects go to _build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libgales_asm.so"
PIPE_RATES = HERE / "pipe_rates"   # arithmetic pipe-rate probe (compute roofline of bench.py)
SOURCES = (["gales_host.cu", "gales_mesh_io.cu", "gales_solver.cu", "gales_magma.cu"] + [f"gales_{t}_{f}.cu" for t in ("hex8", "tet4", "tri3", "quad4") for f in ("fp64", "mixed")]
           + [f"gales_vjp_{t}.cu" for t in ("hex8", "tet4", "tri3", "quad4")]
           + [f"gales_{t}_magma_{f}.cu" for t in ("hex8", "tet4", "tri3", "quad4") for f in ("fp64", "mixed")])
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit contraction in the FP64 form's units, which perform the
# reference's IEEE operations (see gales_physics.cuh); the mixed form's units contract
# freely (the few steps whose rounding must match use unfused intrinsics).
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the GALES library")
    return cand


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "gales_asm.h"]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile (if stale) and return the path of libgales_asm.so."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    jobs = []
    for s in SOURCES:
        src = CSRC / s
        obj = BUILD / (Path(s).stem + ".o")
        if force or _stale(obj, src):
            flags = [("-fmad=true" if (f == "-fmad=false" and "_mixed" in src.name) else f) for f in FLAGS]
            cmd = [nvcc, *ARCH, *flags, "-I", str(HERE.parent / "include"), "-c", str(src), "-o", str(obj)]
            jobs.append((s, cmd))
    pr_src = CSRC / "pipe_rates.cu"
    if force or not PIPE_RATES.exists() or PIPE_RATES.stat().st_mtime < pr_src.stat().st_mtime:
        jobs.append(("pipe_rates.cu", [nvcc, *ARCH, "-std=c++17", "-O3", "-o", str(PIPE_RATES), str(pr_src)]))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): s for s, cmd in jobs}
            for f in cf.as_completed(futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {futs[f]}")
    objs = [str(BUILD / (Path(s).stem + ".o")) for s in SOURCES]
    if force or jobs or not LIB.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("linking libgales_asm.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
