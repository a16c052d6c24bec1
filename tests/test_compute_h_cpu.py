"""compute_h of the mixed form against the reference's operations, checked on the host.

compute_h (gales_physics.cuh) performs quad.hpp:701-739's IEEE operations in their order;
compute_h_fast, the mixed form's version, fuses them, skips the normalisations and, in
3D, takes the third direction's quadratic form from the trace of G where the first two
directions are well conditioned.  Both are compiled here with g++ (contraction off)
behind a small shim for the CUDA intrinsics they call, and compared on random
anisotropic metrics G, velocities and velocity gradients: where compute_h_fast decides
the branch it must agree to 1e-9 relative; where it does not, the kernel falls back to
compute_h.
"""
import ctypes as C
import pathlib
import subprocess

import numpy as np
import pytest

from test_numeric_helpers import _extract

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "gales-multi-fluid_gb300" / "csrc"

SHIM = r"""
#include <cmath>
#define __device__
#define __forceinline__ inline
using std::sqrt; using std::fabs; using std::fma; using std::fmax;
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
constexpr double kEps = 2.220446049250313e-16;
"""


@pytest.fixture(scope="module")
def hlib(tmp_path_factory):
    phys = CSRC / "gales_physics.cuh"
    parts = [SHIM]
    for sig in ("__device__ __forceinline__ double mul_rn(double a, double b)",
                "__device__ __forceinline__ double add_rn(double a, double b)",
                "__device__ __forceinline__ double sub_rn(double a, double b)"):
        parts.append(_extract(phys, sig))
    for sig in ("__device__ __forceinline__ double vsq_rn(const double* v)",
                "__device__ __forceinline__ double compute_h(const double (&G)[DIM][DIM], const double* v,",
                "__device__ __forceinline__ double qform_fma(const double (&G)[DIM][DIM], const double* s)",
                "__device__ __forceinline__ double compute_h_fast(const double (&G)[DIM][DIM], double trG,"):
        parts.append("template <int DIM>\n" + _extract(phys, sig))
    parts.append(r"""
extern "C" void h_many(const double* G, const double* v, const double* dv, long n, double* href, double* hfast,
                       int* decided) {
  for (long i = 0; i < n; ++i) {
    double g[3][3], d[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) { g[a][b] = G[9 * i + 3 * a + b]; d[a][b] = dv[9 * i + 3 * a + b]; }
    const double* vi = v + 3 * i;
    href[i] = compute_h<3>(g, vi, d);
    const double vv = vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2];
    bool dec = false;
    hfast[i] = compute_h_fast<3>(g, g[0][0] + g[1][1] + g[2][2], vi, rsqrt(vv), d, dec);
    decided[i] = dec ? 1 : 0;
  }
}
""")
    d = tmp_path_factory.mktemp("hfast")
    (d / "h.cpp").write_text("\n".join(parts))
    so = d / "h.so"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(so), str(d / "h.cpp")],
                   check=True)
    lib = C.CDLL(str(so))
    lib.h_many.restype = None
    return lib


def _run(lib, G, v, dv):
    n = len(v)
    G, v, dv = (np.ascontiguousarray(x, dtype=np.float64) for x in (G, v, dv))
    href, hfast = np.empty(n), np.empty(n)
    dec = np.empty(n, dtype=np.int32)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    lib.h_many(p(G), p(v), p(dv), C.c_long(n), p(href), p(hfast), p(dec))
    return href, hfast, dec.astype(bool)


def _metrics(rng, n, max_aspect):
    """G = J^-T J^-1-like SPD metrics: random rotations, eigenvalues 1/h_i^2 with
    h_i spread over max_aspect."""
    q, _ = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    h = np.exp(rng.uniform(0.0, np.log(max_aspect), (n, 3))) * 1e-2
    return np.einsum("nij,nj,nkj->nik", q, 1.0 / h ** 2, q)


@pytest.mark.parametrize("max_aspect", [1.0 + 1e-9, 10.0, 1e3])
def test_fast_h_matches_reference_operations(hlib, max_aspect):
    rng = np.random.default_rng(7)
    n = 20000
    G = _metrics(rng, n, max_aspect)
    v = rng.standard_normal((n, 3)) * 0.1
    dv = rng.standard_normal((n, 3, 3))
    href, hfast, dec = _run(hlib, G, v, dv)
    assert dec.mean() > 0.99
    err = np.abs(hfast[dec] - href[dec]) / href[dec]
    assert err.max() <= 1e-9, err.max()


def test_fast_h_near_rank_one_gradients(hlib):
    """dv v nearly parallel to v: |w1| / |dv v| from 1e-2 down to 1e-12, where the trace
    form is not taken and, below 1e-10, the branch is left to compute_h."""
    rng = np.random.default_rng(11)
    n = 6000
    G = _metrics(rng, n, 100.0)
    v = rng.standard_normal((n, 3))
    s0 = v / np.linalg.norm(v, axis=1, keepdims=True)
    t = rng.standard_normal((n, 3))
    t -= np.sum(t * s0, axis=1, keepdims=True) * s0
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    eps = 10.0 ** rng.uniform(-12, -2, n)
    target = s0 + eps[:, None] * t                      # dv v = |v| target
    dv = np.einsum("ni,nj->nij", target, s0)            # dv v = target |v|
    href, hfast, dec = _run(hlib, G, v, dv)
    ok = dec & (eps > 1e-9)
    assert ok.sum() > 0.5 * (eps > 1e-9).sum()
    err = np.abs(hfast[ok] - href[ok]) / href[ok]
    # the reference's own operations move w1's direction by ~1e-16 / eps here
    assert np.all(err <= np.maximum(1e-9, 1e-14 / eps[ok]))
    assert not dec[eps < 1e-11].any()
