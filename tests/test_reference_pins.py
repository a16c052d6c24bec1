"""The oracle pinned against the reference's own code where the reference compiles.

oracle/_ref/libref_classes.so is the reference's chemicals.hpp (custom_chemical, melt,
dissolved_volatiles, ideal_gas over base_chemical.hpp), its
GiordanoEtAlViscosityModel.hpp and its element.hpp (over node.hpp and point.hpp),
compiled from a checkout of the reference by oracle/build.py (build_ref; see
oracle/ref_classes.cpp).  These tests compare the oracle's restatement of the same
quantities with it, on seeded random states where the quantity depends on one:
  - the chemicals' EOS as the assembly's mixture sees them (one-component materials
    built with the package's descriptor constructors, evaluated by the oracle's
    mixture): rho, mu, cp, cv, kappa, sound speed, alpha, beta and the diffusivity;
  - the magma chemicals (Lange-Carmichael melt, dissolved H2O and CO2, the H2O and CO2
    gases) and the Giordano et al. (2008) viscosity, one at a time;
  - the element types' interior Gauss points, side node tables and side Gauss points.
The GPU kernels are compared with the oracle elsewhere (test_gpu_parity.py,
test_magma.py, test_gpu_magma_assembly.py), so these pins close the chain for these
functions.  Skipped where no reference checkout was present at build time.
"""
import ctypes as C
import pathlib

import numpy as np
import pytest

import oracle
from cases import gm

LIB = pathlib.Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libref_classes.so"
KEYS = ["rho", "mu", "cp", "cv", "kappa", "c", "alpha", "beta", "D"]

pytestmark = pytest.mark.skipif(not LIB.exists(), reason="no reference checkout at build time (oracle/_ref)")


@pytest.fixture(scope="module")
def ref():
    lib = C.CDLL(str(LIB))
    d = C.c_double
    dp = C.POINTER(C.c_double)
    lib.ref_custom_chemical.argtypes = [d, d, d, d, d, d, d, d, dp]
    lib.ref_ideal_gas.argtypes = [d, d, d, d, dp]
    lib.ref_ideal_gas_named.argtypes = [C.c_char_p, d, d, dp]
    lib.ref_melt.argtypes = [dp, d, d, d, dp]
    lib.ref_dissolved_volatile.argtypes = [C.c_char_p, d, d, d, d, dp]
    lib.ref_giordano.argtypes = [dp, d, d, d, dp]
    ip = C.POINTER(C.c_int32)
    lib.ref_element_tables.argtypes = [C.c_int, C.c_int, dp, ip, dp, ip]
    return lib


def _out():
    o = np.zeros(9)
    return o, o.ctypes.data_as(C.POINTER(C.c_double))


def _ref_dict(o):
    return dict(zip(KEYS, o))


def _mixture_of_one(chem, p, T):
    """The oracle's mixture (fluid_properties' mix_of_ch) of one chemical."""
    d = oracle.properties(gm.Material([chem]), p, T, np.array([1.0]))
    d["D"] = d["D_c"][0]
    return d


def _close(a, b, rtol):
    return abs(a - b) <= rtol * max(abs(a), abs(b), 1e-300)


@pytest.fixture(scope="module")
def states():
    rng = np.random.default_rng(20261204)
    p = 10 ** rng.uniform(5, 8.3, 60)
    T = rng.uniform(300.0, 1600.0, 60)
    return list(zip(p, T))


def test_custom_chemical_matches_reference(ref, states):
    rng = np.random.default_rng(1)
    for i, (p, T) in enumerate(states):
        rho, mu, cp = rng.uniform(800, 3000), 10 ** rng.uniform(-3, 4), rng.uniform(500, 2500)
        kappa = rng.uniform(0.1, 5.0)
        alpha, beta = (0.0, 0.0) if i % 5 == 0 else (rng.uniform(1e-5, 1e-4), rng.uniform(1e-11, 1e-9))
        o, op = _out()
        ref.ref_custom_chemical(rho, mu, cp, kappa, alpha, beta, p, T, op)
        r = _ref_dict(o)
        m = _mixture_of_one(gm.custom_chemical(rho, mu, cp, kappa, alpha, beta), p, T)
        # stored constants and the component density come through unchanged
        for k in ("mu", "cp", "cv", "kappa", "D"):
            assert m[k] == r[k], (k, m[k], r[k])
        assert m["rho_c"][0] == r["rho"]
        # the one-component mixture's 1/(1/rho), Wood's speed and rho/rho_c weights
        for k in ("rho", "c", "alpha", "beta"):
            assert _close(m[k], r[k], 4e-16), (k, m[k], r[k])


@pytest.mark.parametrize("name", ["H2O", "CO2", "AIR", "HE", "ARGON"])
def test_named_ideal_gas_matches_reference(ref, states, name):
    for p, T in states:
        o, op = _out()
        ref.ref_ideal_gas_named(name.encode(), p, T, op)
        r = _ref_dict(o)
        m = _mixture_of_one(gm.ideal_gas_named(name), p, T)
        for k in ("mu", "cp", "cv", "kappa", "D"):
            assert m[k] == r[k], (name, k, m[k], r[k])
        assert m["rho_c"][0] == r["rho"]
        for k in ("rho", "c", "alpha", "beta"):
            assert _close(m[k], r[k], 4e-16), (name, k, m[k], r[k])


def test_ideal_gas_by_molar_mass_matches_reference(ref, states):
    rng = np.random.default_rng(2)
    for p, T in states:
        M, gamma = rng.uniform(0.002, 0.1), rng.uniform(1.1, 1.7)
        o, op = _out()
        ref.ref_ideal_gas(M, gamma, p, T, op)
        r = _ref_dict(o)
        m = _mixture_of_one(gm.ideal_gas(M, gamma), p, T)
        for k in ("mu", "cp", "cv", "kappa", "D"):
            assert m[k] == r[k], (k, m[k], r[k])
        assert m["rho_c"][0] == r["rho"]
        for k in ("rho", "c", "alpha", "beta"):
            assert _close(m[k], r[k], 4e-16), (k, m[k], r[k])


def _oxides(rng):
    # SiO2 TiO2 Al2O3 Fe2O3 FeO MnO MgO CaO Na2O K2O, unnormalised (both normalise)
    base = np.array([50.0, 1.5, 15.0, 3.0, 7.0, 0.2, 6.0, 10.0, 3.5, 1.5])
    return base * rng.uniform(0.7, 1.3, 10)


def test_magma_chemicals_match_reference(ref, states):
    rng = np.random.default_rng(3)
    for p, T in states:
        wf = _oxides(rng)
        kappa = rng.uniform(0.5, 3.0)
        o, op = _out()
        ref.ref_melt(wf.ctypes.data_as(C.POINTER(C.c_double)), kappa, p, T, op)
        r = _ref_dict(o)
        m = oracle.chemical_props("melt", wf, kappa, p, T)
        for k in ("rho", "cp", "cv", "kappa", "c", "alpha", "beta"):
            assert m[k] == r[k], ("melt", k, m[k], r[k])
        for name, M in (("H2O", 0.01802), ("CO2", 0.04401)):
            cp, kap = rng.uniform(1000, 4000), rng.uniform(0.1, 1.0)
            o, op = _out()
            ref.ref_dissolved_volatile(name.encode(), cp, kap, p, T, op)
            r = _ref_dict(o)
            m = oracle.chemical_props("volatile", M, cp, kap, p, T)
            for k in ("rho", "cp", "cv", "kappa", "c", "alpha", "beta"):
                assert m[k] == r[k], (name, "liquid", k, m[k], r[k])
            o, op = _out()
            ref.ref_ideal_gas_named(name.encode(), p, T, op)
            r = _ref_dict(o)
            m = oracle.chemical_props("gas", M, p, T)
            for k in ("rho", "mu", "cp", "cv", "kappa", "c", "alpha", "beta"):
                assert m[k] == r[k], (name, "gas", k, m[k], r[k])


def test_giordano_viscosity_matches_reference(ref):
    rng = np.random.default_rng(4)
    n_ok = 0
    for _ in range(200):
        wf = _oxides(rng)
        T = rng.uniform(900.0, 1600.0)
        h2o, co2 = rng.uniform(1e-4, 0.06), rng.uniform(0.0, 0.01)
        mu = C.c_double()
        rc = ref.ref_giordano(wf.ctypes.data_as(C.POINTER(C.c_double)), T, h2o, co2, C.byref(mu))
        m = oracle.chemical_props("giordano", wf, T, h2o, co2)
        if rc != 0:
            assert m is None
            continue
        n_ok += 1
        assert m == mu.value, (m, mu.value)
    assert n_ok > 150
    # the reference's error exit (1 - wf_co2_l == 0) is an error in both
    mu = C.c_double()
    wf = _oxides(rng)
    assert ref.ref_giordano(wf.ctypes.data_as(C.POINTER(C.c_double)), 1200.0, 0.01, 1.0, C.byref(mu)) == -1
    assert oracle.chemical_props("giordano", wf, 1200.0, 0.01, 1.0) is None


@pytest.mark.parametrize("dim,nen", [(2, 3), (2, 4), (3, 4), (3, 8)])
def test_element_tables_match_reference(ref, dim, nen):
    """element.hpp's gauss_data: the oracle's (and, through the GPU parity tests, the
    kernels') interior points, side node tables and side points, bit for bit."""
    gp, sgp = np.zeros(8 * 3), np.zeros(6 * 4 * 3)
    sides, cnt = np.zeros(6 * 4, dtype=np.int32), np.zeros(4, dtype=np.int32)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    nq = ref.ref_element_tables(dim, nen, gp.ctypes.data_as(dp), sides.ctypes.data_as(ip), sgp.ctypes.data_as(dp),
                                cnt.ctypes.data_as(ip))
    assert nq > 0
    nq, ns, nsn, nqs = (int(x) for x in cnt)
    o = oracle.gauss(dim, nen)
    assert o["gp"].shape == (nq, 3) and o["sides"].shape == (ns, nsn) and o["sgp"].shape == (ns, nqs, 3)
    assert np.array_equal(o["gp"], gp[:nq * 3].reshape(nq, 3))
    assert np.array_equal(o["sides"], sides[:ns * nsn].reshape(ns, nsn))
    assert np.array_equal(o["sgp"], sgp[:ns * nqs * 3].reshape(ns, nqs, 3))
