"""The point stage's clear of A and b (clear_arrays in gales_kernels.cuh), checked on the
host: its source is compiled with g++ behind a shim that runs it for every thread of a
launch in turn, over arrays at 8- and 16-byte-aligned starts, odd and even lengths and
several grid sizes.  Every word of the range must be zero and the words around it
untouched."""
import ctypes as C
import pathlib
import subprocess

import numpy as np
import pytest

from test_numeric_helpers import _extract

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "gales-multi-fluid_gb300" / "csrc"

SHIM = r"""
#include <cstdint>
#define __device__
#define __forceinline__ inline
struct uint3_ { unsigned x, y, z; };
static uint3_ blockIdx, threadIdx, blockDim, gridDim;
struct double2 { double x, y; };
static inline double2 make_double2(double a, double b) { return {a, b}; }
struct KParams { double* clear_p[2]; int64_t clear_n[2]; };
"""


@pytest.fixture(scope="module")
def clib(tmp_path_factory):
    body = _extract(CSRC / "gales_kernels.cuh", "__device__ __forceinline__ void clear_arrays(const KParams& k)")
    src = SHIM + body + r"""
extern "C" void launch(double* a, long na, double* b, long nb, unsigned grid, unsigned block) {
  KParams k{{a, b}, {na, nb}};
  blockDim = {block, 1, 1};
  gridDim = {grid, 1, 1};
  for (unsigned g = 0; g < grid; ++g)
    for (unsigned t = 0; t < block; ++t) {
      blockIdx = {g, 0, 0};
      threadIdx = {t, 0, 0};
      clear_arrays(k);
    }
}
"""
    d = tmp_path_factory.mktemp("clear")
    (d / "c.cpp").write_text(src)
    so = d / "c.so"
    subprocess.run(["g++", "-O1", "-shared", "-fPIC", "-o", str(so), str(d / "c.cpp")], check=True)
    lib = C.CDLL(str(so))
    lib.launch.restype = None
    lib.launch.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_long, C.c_uint, C.c_uint]
    return lib


def _aligned(n):
    """n NaNs starting on a 16-byte boundary."""
    raw = np.full(n + 2, np.nan)
    s = 0 if raw.ctypes.data % 16 == 0 else 1
    return raw[s:s + n]


@pytest.mark.parametrize("grid,block", [(1, 1), (1, 32), (3, 128), (7, 32)])
def test_clear_covers_exactly_the_range(clib, grid, block):
    for off_a in (0, 1):
        for off_b in (0, 1):
            for na in (0, 1, 2, 3, 16, 17, 1000, 1001):
                nb = (na * 7 + 3) % 41
                A, B = _aligned(na + 4), _aligned(nb + 4)
                clib.launch(A.ctypes.data + 8 * off_a, na, B.ctypes.data + 8 * off_b, nb, grid, block)
                for X, off, n in ((A, off_a, na), (B, off_b, nb)):
                    assert np.all(X[off:off + n] == 0.0)
                    assert np.all(np.isnan(X[:off])) and np.all(np.isnan(X[off + n:]))
