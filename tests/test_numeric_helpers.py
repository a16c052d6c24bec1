"""The integer-only binary64 <-> binary32 conversions of the kernels, checked on the host.

narrow_rn (gales_physics.cuh) and widen (gales_kernels.cuh) replace the hardware
conversion instructions in the mixed form.  Their source is compiled here with g++
behind a small shim for the CUDA bit-cast intrinsics and compared with numpy's IEEE
conversions on special values, overflow, rounding ties, both subnormal ranges and
random bit patterns; narrow_rn flushes results below the smallest normal binary32 to
a signed zero, so those are checked against that rule.
"""
import ctypes as C
import pathlib
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "gales-multi-fluid_gb300" / "csrc"

SHIM = r"""
#include <cstring>
#include <cstdint>
#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long x; std::memcpy(&x, &d, 8); return x; }
static inline double __longlong_as_double(long long x) { double d; std::memcpy(&d, &x, 8); return d; }
static inline unsigned int __float_as_uint(float f) { unsigned int x; std::memcpy(&x, &f, 4); return x; }
static inline float __uint_as_float(unsigned int x) { float f; std::memcpy(&f, &x, 4); return f; }
static inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((unsigned int)x); }
static inline unsigned int __funnelshift_l(unsigned int lo, unsigned int hi, unsigned int s) {
  return (unsigned int)(((((unsigned long long)hi) << 32) | lo) << (s & 31u) >> 32);
}
static inline int __double2hiint(double d) { return (int)(__double_as_longlong(d) >> 32); }
static inline int __double2loint(double d) { return (int)(unsigned int)__double_as_longlong(d); }
static inline double __hiloint2double(int hi, int lo) {
  return __longlong_as_double((long long)(((unsigned long long)(unsigned int)hi << 32) | (unsigned int)lo));
}
"""


def _extract(path, signature):
    text = path.read_text()
    start = text.index(signature)
    depth, i = 0, text.index("{", start)
    while True:
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                return text[start:i + 1]
        i += 1


@pytest.fixture(scope="module")
def conv(tmp_path_factory):
    narrow = _extract(CSRC / "gales_physics.cuh", "__device__ __forceinline__ float narrow_rn(double d)")
    widen = _extract(CSRC / "gales_kernels.cuh", "__device__ __forceinline__ double widen(float f)")
    special = _extract(CSRC / "gales_kernels.cuh", "__device__ __forceinline__ double widen_special(float f) {")
    src = (SHIM + narrow + "\ninline double widen_special(float f);\n" + widen + "\n" + special + r"""
extern "C" void narrow_many(const double* x, float* y, long n) { for (long i = 0; i < n; ++i) y[i] = narrow_rn(x[i]); }
extern "C" void widen_many(const float* x, double* y, long n) { for (long i = 0; i < n; ++i) y[i] = widen(x[i]); }
""")
    d = tmp_path_factory.mktemp("conv")
    (d / "conv.cpp").write_text(src)
    so = d / "conv.so"
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-o", str(so), str(d / "conv.cpp")], check=True)
    lib = C.CDLL(str(so))
    for fn in (lib.narrow_many, lib.widen_many):
        fn.restype = None
    return lib


def _narrow(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(x.shape, dtype=np.float32)
    lib.narrow_many(x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), C.c_long(x.size))
    return y


def _widen(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape, dtype=np.float64)
    lib.widen_many(x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), C.c_long(x.size))
    return y


def _same_bits32(a, b):
    a, b = a.view(np.uint32), b.view(np.uint32)
    nan_a, nan_b = np.isnan(a.view(np.float32)), np.isnan(b.view(np.float32))
    return np.all(nan_a == nan_b) and np.array_equal(a[~nan_a], b[~nan_b])


def test_narrow_matches_ieee(conv):
    rng = np.random.default_rng(0)
    tiny = np.float64(np.finfo(np.float32).smallest_subnormal)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.4028234663852886e38,
                        3.4028235677973366e38, 3.402823669209385e38, 1e39, -1e300, 1.1754943508222875e-38,
                        1.1754942106924411e-38, tiny, tiny * 0.5, tiny * 0.5000001, tiny * 1.5, tiny * 2.5,
                        tiny * 0.49, 1e-46, 5e-324, -5e-324, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24,
                        1.0 + 2.0 ** -24 + 2.0 ** -50])
    bits = rng.integers(0, 2 ** 63, size=400_000, dtype=np.uint64) | (rng.integers(0, 2, 400_000, dtype=np.uint64) << 63)
    randb = bits.view(np.float64)
    # values near the float range and its subnormals
    near = np.concatenate([rng.uniform(-1, 1, 100_000) * 10.0 ** rng.uniform(-46, 39, 100_000),
                           (rng.integers(1, 2 ** 23, 50_000) * tiny) * (1 + rng.uniform(-1e-7, 1e-7, 50_000))])
    for x in (special, randb, near):
        with np.errstate(over="ignore", invalid="ignore"):
            ref = x.astype(np.float32)
        # results below the smallest normal flush to a signed zero
        sub = np.abs(ref) < np.finfo(np.float32).tiny
        ref[sub] = np.copysign(np.float32(0.0), ref[sub])
        # inputs that round up to the smallest normal but lie below it flush as well
        low = np.abs(x) < np.float64(np.finfo(np.float32).tiny)
        ref[low] = np.copysign(np.float32(0.0), x[low]).astype(np.float32)
        assert _same_bits32(_narrow(conv, x), ref)


def test_widen_is_exact(conv):
    rng = np.random.default_rng(1)
    bits = rng.integers(0, 2 ** 32, size=400_000, dtype=np.uint64).astype(np.uint32)
    x = np.concatenate([bits.view(np.float32),
                        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1.1754942e-38,
                                  3.4028235e38], dtype=np.float32)])
    y = _widen(conv, x)
    with np.errstate(invalid="ignore"):
        ref = x.astype(np.float64)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(y), nan)
    assert np.array_equal(y[~nan].view(np.uint64), ref[~nan].view(np.uint64))
