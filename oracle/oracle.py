"""TEST INFRASTRUCTURE — ctypes binding of the CPU oracle (gales_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this,
as the checker.  PARITY UNPINNED for the assembly: the reference's element integral
cannot be built here (Boost, MPI and Trilinos are absent) and it ships no golden data;
its chemicals and magma viscosity model compile, and the oracle is pinned against them
(tests/test_reference_pins.py); see the header of gales_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import importlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(HERE) not in sys.path:
    sys.path.insert(0, str(HERE))

import build as _build  # noqa: E402  (oracle/build.py)

gm = importlib.import_module("gales-multi-fluid_gb300")
abi = gm.abi

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        vp, dp, i64p, i32p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32)
        L.gor_properties.argtypes = [C.POINTER(abi.MaterialDesc), C.c_double, C.c_double, dp, dp]
        L.gor_inverse.argtypes = [C.c_int, dp, dp]
        L.gor_quad.argtypes = [C.c_int, C.c_int, dp, dp, C.c_int, dp]
        L.gor_gauss.argtypes = [C.c_int, C.c_int, dp, i32p, dp, i32p]
        L.gor_pattern_count.argtypes = [C.POINTER(abi.MeshDesc), C.c_int, i64p]
        L.gor_pattern_count.restype = C.c_int64
        L.gor_pattern.argtypes = [C.POINTER(abi.MeshDesc), C.c_int, i64p, i32p, i64p, i32p]
        L.gor_colouring.argtypes = [C.POINTER(abi.MeshDesc), i32p, i32p]
        L.gor_element.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(abi.MaterialDesc), C.POINTER(abi.SetupDesc),
                                  dp, dp, C.c_double, C.c_int64, C.c_int, dp, dp]
        L.gor_assemble.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(abi.MaterialDesc), C.POINTER(abi.SetupDesc),
                                   dp, dp, C.c_double, i64p, i32p, dp, dp, C.c_int, i32p, C.c_int32, i64p]
        L.gor_adaptive_dt.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(abi.MaterialDesc),
                                      C.POINTER(abi.SetupDesc), dp, C.c_double, C.c_double, dp]
        L.gor_iluk.argtypes = [C.c_int64, i64p, i32p, dp, C.c_int32, i64p, i64p, i32p, dp]
        L.gor_iluk.restype = C.c_int64
        L.gor_fgmres.argtypes = [C.c_int64, i64p, i32p, dp, dp, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                 C.c_int32, C.c_int64, dp, dp]
        L.gor_fgmres.restype = C.c_int64
        L.gor_magma_properties.argtypes = [C.POINTER(abi.MagmaDesc), C.c_int32, dp, dp, dp, dp, C.c_int64, dp, dp]
        L.gor_magma_properties.restype = C.c_int
        L.gor_set_magma.argtypes = [C.POINTER(abi.MagmaDesc), C.c_int32]
        L.gor_set_magma.restype = C.c_int
        L.gor_shear_rate.argtypes = [C.c_int, dp]
        L.gor_shear_rate.restype = C.c_double
        L.gor_magma_fractions.argtypes = [C.c_double, C.c_double, dp, dp]
        L.gor_magma_fractions.restype = C.c_int
        for f in ("gor_properties", "gor_inverse", "gor_quad", "gor_gauss", "gor_pattern", "gor_colouring",
                  "gor_element", "gor_assemble", "gor_adaptive_dt"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i64(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _i32(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def properties(material, p, T, Y):
    nc = material.nb_comp
    out = np.zeros(9 + 3 * nc)
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    lib().gor_properties(C.byref(material.desc), p, T, _d(Y), _d(out))
    keys = ["rho", "mu", "cp", "cv", "kappa", "D", "c", "alpha", "beta"]
    d = dict(zip(keys, out[:9]))
    d["rho_c"] = out[9::3].copy()
    d["e_c"] = out[10::3].copy()
    d["D_c"] = out[11::3].copy()
    return d


def inverse(A):
    A = np.ascontiguousarray(A, dtype=np.float64)
    n = A.shape[0]
    inv = np.zeros_like(A)
    s = lib().gor_inverse(n, _d(A), _d(inv))
    return inv, s


def quad(dim, nen, xe, pt, boundary=False):
    xe = np.ascontiguousarray(xe, dtype=np.float64)
    pt = np.ascontiguousarray(pt, dtype=np.float64)
    out = np.zeros(nen + dim * nen + 2 + dim * dim + 2 * dim)
    rc = lib().gor_quad(dim, nen, _d(xe), _d(pt), int(boundary), _d(out))
    o = 0
    sh = out[o:o + nen]; o += nen
    ds = out[o:o + dim * nen].reshape(dim, nen); o += dim * nen
    J, JxW = out[o], out[o + 1]; o += 2
    G = out[o:o + dim * dim].reshape(dim, dim); o += dim * dim
    g = out[o:o + dim]; o += dim
    JNxW = out[o:o + dim]
    return dict(sh=sh, ds=ds, J=J, JxW=JxW, G=G, g=g, JNxW=JNxW, status=rc)


def gauss(dim, nen):
    gp = np.zeros(8 * 3)
    sides = np.zeros(6 * 4, dtype=np.int32)
    sgp = np.zeros(6 * 4 * 3)
    cnt = np.zeros(4, dtype=np.int32)
    lib().gor_gauss(dim, nen, _d(gp), _i32(sides), _d(sgp), _i32(cnt))
    nq, ns, nsn, nqs = (int(x) for x in cnt)
    return dict(gp=gp[:nq * 3].reshape(nq, 3), sides=sides[:ns * nsn].reshape(ns, nsn),
                sgp=sgp[:ns * nqs * 3].reshape(ns, nqs, 3))


def pattern(mesh, nd, scalar=True):
    nnz_nodes = C.c_int64()
    nnz = lib().gor_pattern_count(C.byref(mesh.desc()), nd, C.byref(nnz_nodes))
    nrp = np.zeros(mesh.n_nodes + 1, dtype=np.int64)
    ncol = np.zeros(nnz_nodes.value, dtype=np.int32)
    if scalar:
        rp = np.zeros(mesh.n_nodes * nd + 1, dtype=np.int64)
        col = np.zeros(nnz, dtype=np.int32)
        lib().gor_pattern(C.byref(mesh.desc()), nd, _i64(nrp), _i32(ncol), _i64(rp), _i32(col))
        return nrp, ncol, rp, col
    lib().gor_pattern(C.byref(mesh.desc()), nd, _i64(nrp), _i32(ncol), None, None)
    return nrp, ncol, None, None


def colouring(mesh):
    colour = np.zeros(mesh.n_elements, dtype=np.int32)
    nc = C.c_int32()
    lib().gor_colouring(C.byref(mesh.desc()), _i32(colour), C.byref(nc))
    return colour, nc.value


def element(mesh, material, setup, I, P, dt, e, which=0, want_matrix=True):
    nd = gm.nb_dofs(mesh.dim, material.nb_comp)
    n = mesh.nen * nd
    m = np.zeros((n, n)) if want_matrix else None
    r = np.zeros(n)
    I = np.ascontiguousarray(I, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    s = lib().gor_element(C.byref(mesh.desc()), C.byref(material.desc), C.byref(setup.desc), _d(I), _d(P), dt, e,
                          which, _d(m) if want_matrix else None, _d(r))
    return m, r, s


def assemble(mesh, material, setup, I, P, dt, row_ptr, col, want_matrix=True, nthreads=1, colour=None,
             n_colours=0):
    """fluid_assembly::execute on the CPU: returns (vals, rhs, status, first_bad)."""
    I = np.ascontiguousarray(I, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    vals = np.zeros(int(row_ptr[-1])) if want_matrix else None
    rhs = np.zeros(len(row_ptr) - 1)
    fb = C.c_int64(-1)
    colour_p = None
    if colour is not None:
        colour = np.ascontiguousarray(colour, dtype=np.int32)
        colour_p = _i32(colour)
    s = lib().gor_assemble(C.byref(mesh.desc()), C.byref(material.desc), C.byref(setup.desc), _d(I), _d(P), dt,
                           _i64(row_ptr), _i32(col), _d(vals) if want_matrix else None, _d(rhs), nthreads, colour_p,
                           n_colours, C.byref(fb))
    return vals, rhs, s, fb.value


def adaptive_dt(mesh, material, setup, I, dt, cfl):
    """adaptive_time_criteria::f_mc on the CPU: every element's smallest Gauss-point dt."""
    I = np.ascontiguousarray(I, dtype=np.float64)
    out = np.zeros(mesh.n_elements)
    s = lib().gor_adaptive_dt(C.byref(mesh.desc()), C.byref(material.desc), C.byref(setup.desc), _d(I),
                              float(dt), float(cfl), _d(out))
    if s:
        raise RuntimeError(f"gor_adaptive_dt status {s}")
    return out


def set_dt(dt_el_min, dt, dt_min, dt_max):
    """set_dt (adaptive_time_step.hpp:380-393)."""
    d = 1.01 * dt if dt_el_min > 1.01 * dt else dt_el_min
    return max(min(d, dt_max), dt_min)


def iluk(row_ptr, col, vals, fill=1):
    """Ifpack ILU(fill) of a CSR matrix (solver_oracle.cpp): (f_rp, f_col, f_val, bad_row)."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    n = len(row_ptr) - 1
    nnz = C.c_int64()
    lib().gor_iluk(n, _i64(row_ptr), _i32(col), _d(vals), int(fill), C.byref(nnz), None, None, None)
    f_rp = np.zeros(n + 1, dtype=np.int64)
    f_col = np.zeros(nnz.value, dtype=np.int32)
    f_val = np.zeros(nnz.value)
    bad = lib().gor_iluk(n, _i64(row_ptr), _i32(col), _d(vals), int(fill), C.byref(nnz), _i64(f_rp), _i32(f_col),
                         _d(f_val))
    return f_rp, f_col, f_val, int(bad) - 1


def fgmres(row_ptr, col, vals, b, tol=1e-9, maxsubspace=200, maxrestarts=5, maxiters=-1, fill=1, precond=True):
    """belos_linear_solver::execute with Flexible GMRES and ILU (solver_oracle.cpp).
    Returns (x, dict(iterations, abs_res, rel_res, converged, cycles))."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = len(row_ptr) - 1
    x = np.zeros(n)
    out = np.zeros(5)
    bad = lib().gor_fgmres(n, _i64(row_ptr), _i32(col), _d(vals), _d(b), int(fill), int(bool(precond)), float(tol),
                           int(maxsubspace), int(maxrestarts), int(maxiters), _d(x), _d(out))
    if bad:
        raise ZeroDivisionError(f"zero pivot in row {bad - 1}")
    return x, dict(iterations=int(out[0]), abs_res=float(out[1]), rel_res=float(out[2]), converged=bool(out[3]),
                   cycles=int(out[4]))


def magma_properties(comps, p, T, Y, shear=None):
    """fluid_properties' mix_of_mix of magma mixtures on the CPU (magma_oracle.cpp):
    (out[8, n], comp[nc, 4, n], status bits)."""
    magma = importlib.import_module("gales-multi-fluid_gb300.magma")
    arr = magma.descs(comps)
    p = np.ascontiguousarray(p, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    n = len(p)
    out = np.zeros((8, n))
    comp = np.zeros((len(comps), 4, n))
    sh = None if shear is None else np.ascontiguousarray(shear, dtype=np.float64)
    st = lib().gor_magma_properties(arr, len(comps), _d(p), _d(T), _d(Y), _d(sh) if sh is not None else None, n,
                                    _d(out), _d(comp))
    return out, comp, int(st)


class magma_material:
    """Context manager: the oracle's assembly, element and property calls use the given
    magma mixtures (mix_of_mix) instead of the material's chemicals."""

    def __init__(self, comps):
        magma = importlib.import_module("gales-multi-fluid_gb300.magma")
        self._comps = list(comps)  # owns the tables the descriptors point to
        self._arr = magma.descs(self._comps)
        self._n = len(comps)

    def __enter__(self):
        lib().gor_set_magma(self._arr, self._n)
        return self

    def __exit__(self, *exc):
        lib().gor_set_magma(None, 0)
        return False


def shear_rate(dim, dI):
    """compute_shear_rate (non_newtonian.hpp:23-39) from dI[k][j] = dI_j/dx_k, shape
    (3, GALES_MAX_ND)."""
    dI = np.ascontiguousarray(dI, dtype=np.float64)
    return float(lib().gor_shear_rate(int(dim), _d(dI)))


def chemical_props(kind, *args):
    """One restated chemical or the viscosity model (magma_oracle.cpp), for the pins
    against the reference's classes: kind "melt" (oxide_wf[10], kappa, p, T), "volatile"
    (molar_mass, cp, kappa, p, T), "gas" (molar_mass, p, T) -> dict of rho, mu, cp, cv,
    kappa, c, alpha, beta, D; "giordano" (oxide_wf[10], T, wf_h2o_l, wf_co2_l) -> mu or
    None on the reference's error exits."""
    out = np.zeros(9)
    L = lib()
    if kind == "melt":
        wf, kappa, p, T = args
        L.gor_melt_props(_d(np.ascontiguousarray(wf, dtype=np.float64)), C.c_double(kappa), C.c_double(p),
                         C.c_double(T), _d(out))
    elif kind == "volatile":
        M, cp, kappa, p, T = args
        L.gor_volatile_props(*(C.c_double(x) for x in (M, cp, kappa, p, T)), _d(out))
    elif kind == "gas":
        M, p, T = args
        L.gor_gas_props(*(C.c_double(x) for x in (M, p, T)), _d(out))
    elif kind == "giordano":
        wf, T, h2o, co2 = args
        mu = C.c_double()
        r = L.gor_giordano_mu(_d(np.ascontiguousarray(wf, dtype=np.float64)), *(C.c_double(x) for x in (T, h2o, co2)),
                              C.byref(mu))
        return None if r else mu.value
    else:
        raise ValueError(kind)
    return dict(zip(["rho", "mu", "cp", "cv", "kappa", "c", "alpha", "beta", "D"], out))


def magma_fractions(p, T, Y):
    """secondary_dofs::execute's gas fractions (pp_vf_g, secondary_dofs.hpp:56-131) with
    the magmas set by magma_material, at points (p[i], T[i], Y[i, :]): (2 nc + 6, n)."""
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    n, nc = Y.shape
    out = np.zeros((n, 2 * nc + 6))
    for i in range(n):
        st = lib().gor_magma_fractions(float(p[i]), float(T[i]), _d(Y[i]), _d(out[i]))
        if st < 0:
            raise RuntimeError("no magma material set")
    return out.T.copy()


def pressure_profile(material, p0, h, T, T1, Y, Y1):
    """pressure_profile_mc::Runge_Kutta (pressure_profile.hpp:480-496), with the last
    mass fraction formed as 1 - accumulate(...) (pressure_profile.hpp:378-388)."""
    nc = material.nb_comp
    n = len(T) - 1

    def full(y):
        s = 0.0
        for c in range(nc - 1):
            s = s + float(y[c])
        return [float(x) for x in y[:nc - 1]] + [1.0 - s]

    def rho(p, t, y):
        return properties(material, p, t, np.asarray(full(y)))["rho"]

    p = [float(p0)]
    for i in range(n):
        m1 = 9.81 * rho(p[i], T[i], Y[i])
        m2 = 9.81 * rho(p[i] + 0.5 * h * m1, T1[i], Y1[i])
        m3 = 9.81 * rho(p[i] + 0.5 * h * m2, T1[i], Y1[i])
        m4 = 9.81 * rho(p[i] + h * m3, T[i + 1], Y[i + 1])
        p.append(p[i] + h / 6. * (m1 + 2.0 * (m2 + m3) + m4))
    return np.array(p)


def pressure_interpolate(y_col, p_col, y):
    """p_interpolation (pressure_profile.hpp:26-41)."""
    import bisect
    y_col = [float(v) for v in y_col]
    out = []
    for yy in y:
        if y_col[0] < y_col[-1]:
            i = bisect.bisect_left(y_col, yy)
        else:
            neg = [-v for v in y_col]
            i = bisect.bisect_left(neg, -yy)
        if i > 0:
            i -= 1
        if i >= len(y_col) - 1:
            raise IndexError("index i goes out of the vector scope")
        f = (yy - y_col[i]) / (y_col[i + 1] - y_col[i])
        out.append(f * p_col[i + 1] + (1.0 - f) * p_col[i])
    return np.array(out)
