"""Magma mixtures (mixtures.hpp:114-511, the props.txt mix_of_mix of magma_mix of the
shipped cases): lookup-table interpolation, the five chemicals, Giordano viscosity, the
gas and crystal corrections and the mixture of sub-mixtures (fluid_properties.hpp:
171-200).

CPU: the kernel's code (gales_magma.cuh) compiled for the host equals the oracle
(magma_oracle.cpp) bit for bit; properties are physically consistent; props.txt and the
lookup-table files parse.  GPU: the kernel against the oracle within the differences of
the CUDA and host math libraries.
"""
import ctypes as C
import importlib
import os
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = pathlib.Path(__file__).resolve().parents[1]
gm = importlib.import_module("gales-multi-fluid_gb300")
magma = importlib.import_module("gales-multi-fluid_gb300.magma")
syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")

MODELS = [("Ishii_Zuber", "none", 0.0, 0), ("none", "Einstein_Roscoe", 0.2, 0), ("none", "Caricchi", 0.3, 0),
          ("Pal_2003", "none", 0.0, 0), ("Ishii_Zuber", "Caricchi", 0.1, 7), ("none", "none", 0.0, 7)]


def _points(n=257, seed=0, nc=2):
    rng = np.random.default_rng(seed)
    p = rng.uniform(6.05e7, 2.995e8, n)
    T = rng.uniform(1120.0, 1480.0, n)
    Y = rng.dirichlet(np.ones(nc), n)
    shear = rng.uniform(0.0, 20.0, n)
    shear[::5] = 0.0
    return p, T, Y, shear


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not found")
    so = tmp_path_factory.mktemp("magma") / "magma_host.so"
    subprocess.run(["nvcc", "-std=c++17", "-O1", "-x", "cu", "-shared", "-Xcompiler", "-fPIC", "-Xcompiler",
                    "-ffp-contract=off", "-o", str(so), str(ROOT / "tests" / "host" / "magma_host.cu")], check=True)
    L = C.CDLL(str(so))
    dp = C.POINTER(C.c_double)
    L.magma_host_properties.argtypes = [C.POINTER(gm.abi.MagmaDesc), C.c_int32, dp, dp, dp, dp, C.c_int64, dp, dp]
    L.magma_host_properties.restype = C.c_int
    L.magma_host_fractions.argtypes = [C.POINTER(gm.abi.MagmaDesc), C.c_int32, dp, dp, dp, C.c_int64, dp]
    L.magma_host_fractions.restype = C.c_int
    return L


def _host(L, comps, p, T, Y, shear):
    d = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    n, nc = len(p), len(comps)
    out = np.zeros((8, n))
    comp = np.zeros((nc, 4, n))
    Y = np.ascontiguousarray(Y)
    st = L.magma_host_properties(magma.descs(comps), nc, d(p), d(T), d(Y), d(shear) if shear is not None else None,
                                 n, d(out), d(comp))
    return out, comp, st


@pytest.mark.parametrize("gas, crystal, cf, n_T", MODELS)
def test_kernel_code_equals_oracle_on_host(gas, crystal, cf, n_T, host_lib):
    comps = syn.magma_pair(gas, crystal, cf, n_T=n_T)
    p, T, Y, shear = _points()
    o1, c1, s1 = _host(host_lib, comps, p, T, Y, shear)
    o2, c2, s2 = oracle.magma_properties(comps, p, T, Y, shear)
    assert s1 == s2 == 0
    assert np.array_equal(o1, o2, equal_nan=True) and np.array_equal(c1, c2, equal_nan=True)


@pytest.mark.parametrize("n_T", [0, 7])
def test_gas_fractions_kernel_code_equals_oracle(n_T, host_lib):
    """secondary_dofs' pp_vf_g fractions (secondary_dofs.hpp:113-131): the kernel's code on
    the host equals the oracle bit for bit, and the totals agree with the mixture's own
    outputs (vf_g_on_total = sum_c Y_c rho / rho_c vf_gas_c)."""
    comps = syn.magma_pair(n_T=n_T)
    p, T, Y, _ = _points()
    n, nc = len(p), len(comps)
    got = np.zeros((2 * nc + 6, n))
    d = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    Yc = np.ascontiguousarray(Y)
    st = host_lib.magma_host_fractions(magma.descs(comps), nc, d(p), d(T), d(Yc), n, d(got))
    with oracle.magma_material(comps):
        ref = oracle.magma_fractions(p, T, Y)
    assert st == 0 and np.array_equal(got, ref)
    out, comp, _ = oracle.magma_properties(comps, p, T, Y)
    vf = sum(Y[:, c] * out[0] / comp[c, 0] * comp[c, 3] for c in range(nc))
    np.testing.assert_allclose(ref[2 * nc], vf, rtol=1e-13)
    np.testing.assert_allclose(ref[2 * nc], ref[2 * nc + 1] + ref[2 * nc + 2], rtol=1e-12)
    assert np.all((ref[2 * nc + 3] > 0) & (ref[2 * nc + 3] < 1))


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_shear_rate_formula(dim):
    """compute_shear_rate (non_newtonian.hpp:23-29, 32-39), which the magma viscosity
    models read at I and at the boundary points: sqrt(u_x^2 + v_y^2 (+ w_z^2)
    + 2 (u_y + v_x)^2 (+ 2 (u_z + w_x)^2 + 2 (v_z + w_y)^2)), from dI[k][j] = dI_j/dx_k."""
    rng = np.random.default_rng(dim)
    for _ in range(20):
        dI = np.zeros((3, gm.abi.MAX_ND))
        dI[:dim, :] = rng.normal(size=(dim, gm.abi.MAX_ND))
        g = dI[:dim, 1:1 + dim].T          # g[i][j] = d v_i / d x_j
        if dim == 2:
            ref = np.sqrt(g[0, 0] ** 2 + g[1, 1] ** 2 + 2 * (g[0, 1] + g[1, 0]) ** 2)
        else:
            ref = np.sqrt(g[0, 0] ** 2 + g[1, 1] ** 2 + g[2, 2] ** 2 + 2 * (g[0, 1] + g[1, 0]) ** 2
                          + 2 * (g[0, 2] + g[2, 0]) ** 2 + 2 * (g[1, 2] + g[2, 1]) ** 2)
        assert oracle.shear_rate(dim, dI) == pytest.approx(ref, rel=1e-15)


def _with_submixtures(kind):
    """Mixtures of sub-mixtures of every kind: magma_mix, custom_mix, ch_as_mix."""
    mg = syn.magma_pair()[0]
    melt = magma.CustomMix("melt", rho=2400.0, mu=1.0e3, cp=1200.0, kappa=1.5, alpha=3e-5, beta=1e-10)
    rigid = magma.CustomMix("rigid", rho=2700.0, mu=1.0e4, cp=1000.0, kappa=2.0)
    gas = magma.ChemicalAsMix("h2o", gm.ideal_gas_named("H2O"))
    liquid = magma.ChemicalAsMix("liq", gm.custom_chemical(rho=2300.0, mu=500.0, cp=1100.0, kappa=1.2, alpha=2e-5,
                                                           beta=2e-10))
    return {"magma+custom": [mg, melt], "magma+gas": [mg, gas], "custom+chemical": [rigid, liquid],
            "three": [mg, liquid, gas]}[kind]


@pytest.mark.parametrize("kind", ["magma+custom", "magma+gas", "custom+chemical", "three"])
def test_submixture_kinds_kernel_code_equals_oracle(kind, host_lib):
    """custom_mix (mixtures.hpp:69-101) and ch_as_mix (mixtures.hpp:25-53) beside magma_mix
    in a mix_of_mix: the kernel's code on the host equals the oracle bit for bit."""
    comps = _with_submixtures(kind)
    p, T, Y, shear = _points(nc=len(comps))
    o1, c1, s1 = _host(host_lib, comps, p, T, Y, shear)
    o2, c2, s2 = oracle.magma_properties(comps, p, T, Y, shear)
    assert s1 == s2 == 0
    assert np.array_equal(o1, o2) and np.array_equal(c1, c2)


def test_custom_mix_closed_forms():
    """custom_mixture: constant rho, mu, cp, kappa; sound speed 1/sqrt(rho beta) (1e20 for
    beta = 0); cv = cp - T alpha^2/(rho beta) (cp for beta = 0); diffusivity 1e-10."""
    cm = magma.CustomMix("m", rho=2400.0, mu=1.0e3, cp=1200.0, kappa=1.5, alpha=3e-5, beta=1e-10)
    rigid = magma.CustomMix("r", rho=2700.0, mu=1.0e4, cp=1000.0, kappa=2.0)
    T = np.array([1200.0, 1300.0])
    out, comp, st = oracle.magma_properties([cm], np.full(2, 1e8), T, np.ones((2, 1)))
    assert st == 0
    np.testing.assert_allclose(out[0], 2400.0, rtol=0)
    np.testing.assert_allclose(out[5], 1.0 / np.sqrt(2400.0 * 1e-10), rtol=1e-15)
    np.testing.assert_allclose(out[3], 1200.0 - T * 9e-10 / (2400.0 * 1e-10), rtol=1e-15)
    assert np.all(comp[0, 2] == 1e-10) and np.all(comp[0, 3] == 0.0)
    out, comp, st = oracle.magma_properties([rigid], np.full(2, 1e8), T, np.ones((2, 1)))
    assert np.all(out[3] == 1000.0) and np.all(out[5] == 1e20)


def test_chemicals_as_submixtures_equal_the_mixture_of_chemicals():
    """A mix_of_mix of ch_as_mix sub-mixtures (fluid_properties.hpp:171-200) is the
    mix_of_ch of the same chemicals (fluid_properties.hpp:199-227): the same properties
    and the same assembled system in the oracle (the mixtures' own diffusivities are not
    read by the assembly; the components' are 1e-10 in both)."""
    mat = syn.material_for(3, 0)
    comps = [magma.ChemicalAsMix(f"c{i}", q) for i, q in enumerate(mat.chemicals)]
    mesh = syn.box_tet_delaunay(4, seed=2)
    setup = syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, 0)
    nrp, ncol, rp, col = oracle.pattern(mesh, 7)
    v0, r0, s0, _ = oracle.assemble(mesh, mat, setup, I, P, 1e-3, rp, col)
    with oracle.magma_material(comps):
        v1, r1, s1, _ = oracle.assemble(mesh, mat, setup, I, P, 1e-3, rp, col)
    assert s0 == s1 == 0
    assert np.linalg.norm(v1 - v0) <= 1e-14 * np.linalg.norm(v0)
    assert np.linalg.norm(r1 - r0) <= 1e-14 * np.linalg.norm(r0)


def test_physical_consistency():
    """rho of the mixture of sub-mixtures is the harmonic Y-average of the components';
    the gas volume fraction grows as the pressure falls; Ishii-Zuber divides mu by
    1 - vf_gas; Einstein-Roscoe multiplies it by (1 - phi)^-2.5."""
    p, T, Y, shear = _points(64)
    out, comp, st = oracle.magma_properties(syn.magma_pair("none"), p, T, Y)
    assert st == 0
    rho_c = comp[:, 0]
    assert np.allclose(out[0], 1.0 / (Y.T / rho_c).sum(0), rtol=1e-14)
    assert np.all((comp[:, 3] >= 0) & (comp[:, 3] < 0.5))
    assert np.all((out[0] > 2000) & (out[0] < 3000)) and np.all(out[1] > 1.0) and np.all(out[5] > 100.0)
    # degassing: the gas volume fraction grows as the pressure falls
    ps = np.linspace(2.99e8, 6.1e7, 40)
    _, c_p, _ = oracle.magma_properties(syn.magma_pair("none"), ps, np.full(40, 1300.0), np.full((40, 2), 0.5))
    assert np.all(np.diff(c_p[:, 3], axis=1) > 0)
    oi, ci, _ = oracle.magma_properties(syn.magma_pair("Ishii_Zuber")[:1], p, T, np.ones((64, 1)))
    on, cn, _ = oracle.magma_properties(syn.magma_pair("none")[:1], p, T, np.ones((64, 1)))
    assert np.allclose(oi[1], on[1] / (1.0 - cn[0, 3]), rtol=1e-14)
    oe, _, _ = oracle.magma_properties(syn.magma_pair("none", "Einstein_Roscoe", 0.2)[:1], p, T, np.ones((64, 1)))
    oc, cc, _ = oracle.magma_properties(syn.magma_pair("none", "none", 0.2)[:1], p, T, np.ones((64, 1)))
    assert np.allclose(oe[1], oc[1] * 0.8 ** -2.5, rtol=1e-14)


def test_pal_2003_iteration_reproduces_the_reference_loop():
    """Pal 2003 (mixtures.hpp:260-291) iterates while F < 1e-9 from x = 1e-5: the first
    Newton step leaves far past the root and the result is NaN for these states, in the
    restatement as in the reference; with zero shear the correction is skipped."""
    p, T, Y, shear = _points(16)
    o, _, st = oracle.magma_properties(syn.magma_pair("Pal_2003"), p, T, Y, np.full(16, 1.0))
    assert st == 0 and np.all(np.isnan(o[1]))
    o0, _, _ = oracle.magma_properties(syn.magma_pair("Pal_2003"), p, T, Y, np.zeros(16))
    on, _, _ = oracle.magma_properties(syn.magma_pair("none"), p, T, Y, np.zeros(16))
    assert np.array_equal(o0[1], on[1])


def test_out_of_table_is_reported():
    out, comp, st = oracle.magma_properties(syn.magma_pair(), np.array([5.0e7, 3.5e8]), np.array([1300.0, 1300.0]),
                                            np.full((2, 2), 0.5))
    assert st == gm.abi.MAGMA_LOOKUP_RANGE


PROPS = """fluid
{
     mix_of_mix
     {
        magma_mix
        {
            name                  basaltic
            oxide_wf              0.49, 0.015, 0.16, 0.02, 0.08, 0.002, 0.08, 0.11, 0.03, 0.013

            h2o_wf                0.02
            co2_wf                0.01
            crystal_fraction      0.1
            crystal_rho           2700.0
            gas_on_mu_model       Ishii_Zuber
            crystal_on_mu_model   Caricchi
        }

        magma_mix
        {
            name                  trachytic
            oxide_wf              0.6, 0.005, 0.18, 0.02, 0.03, 0.001, 0.01, 0.03, 0.06, 0.06
            melt_kappa            1.2
            h2o_wf                0.01
            co2_wf                0.001
            gas_on_mu_model       Ishii_Zuber
            crystal_on_mu_model   none
        }
     }
}
"""


def test_read_props_and_lookup_tables(tmp_path):
    (tmp_path / "props.txt").write_text(PROPS)
    mixes = magma.read_props(tmp_path / "props.txt")
    assert [m.name for m in mixes] == ["basaltic", "trachytic"]
    a, b = mixes
    assert a.oxide_wf[0] == 0.49 and a.h2o_wf == 0.02 and a.crystal_fraction == 0.1 and a.crystal_rho == 2700.0
    assert a.gas_on_mu == "Ishii_Zuber" and a.crystal_on_mu == "Caricchi"
    assert b.melt_kappa == 1.2 and b.h2o_l_cp == 2278.0 and b.crystal_on_mu == "none"
    ref = syn.magma_pair(n_T=5)
    for m, r in zip(mixes, ref):
        m.name = r.name
        r_dir = tmp_path / "lookuptable"
        magma.write_lookup_tables(r_dir, r)
        magma.read_lookup_tables(r_dir, m)
        assert np.array_equal(m.p_table, r.p_table) and np.array_equal(m.T_table, r.T_table)
        assert np.array_equal(m.wf_l_h2o, r.wf_l_h2o.ravel()) and np.array_equal(m.wf_l_co2, r.wf_l_co2.ravel())
    with pytest.raises(ValueError):
        (tmp_path / "bad.txt").write_text("fluid\n{\n  custom_mix\n  {\n  }\n}\n")
        magma.read_props(tmp_path / "bad.txt")


# ---------------------------------------------------------------------------
# GPU


@pytest.mark.gpu
@pytest.mark.parametrize("gas, crystal, cf, n_T", MODELS)
def test_gpu_matches_oracle(gas, crystal, cf, n_T, cuda_lib):
    comps = syn.magma_pair(gas, crystal, cf, n_T=n_T)
    mat = magma.MagmaMaterial(comps)
    p, T, Y, shear = _points(1000, seed=1)
    got = mat.properties(p, T, Y, shear, with_components=True)
    ref, comp, st = oracle.magma_properties(comps, p, T, Y, shear)
    assert st == 0
    for k, name in enumerate(magma.FIELDS):
        np.testing.assert_allclose(got[name], ref[k], rtol=1e-12, atol=0, equal_nan=True, err_msg=name)
    for k, name in enumerate(magma.COMP_FIELDS):
        np.testing.assert_allclose(got["comp_" + name], comp[:, k], rtol=1e-12, atol=1e-300, equal_nan=True,
                                   err_msg=name)


@pytest.mark.gpu
def test_gpu_device_buffers_and_range_status(cuda_lib):
    import torch
    comps = syn.magma_pair()
    mat = magma.MagmaMaterial(comps)
    p, T, Y, shear = _points(300, seed=2)
    dev = "cuda:0"
    got = mat.properties(torch.tensor(p, device=dev), torch.tensor(T, device=dev), torch.tensor(Y, device=dev))
    ref, _, _ = oracle.magma_properties(comps, p, T, Y)
    np.testing.assert_allclose(got["rho"].cpu().numpy(), ref[0], rtol=1e-12)
    np.testing.assert_allclose(got["mu"].cpu().numpy(), ref[1], rtol=1e-12)
    with pytest.raises(gm.GalesError):
        mat.properties(np.array([5.0e7, 1.0e8]), np.array([1300.0, 1300.0]), np.full((2, 2), 0.5))
    assert gm.abi.lib().gales_magma_status(mat._h) == gm.abi.MAGMA_LOOKUP_RANGE


def test_oracle_assembly_with_magma_material():
    """The oracle's assembly with the chemicals replaced by two magma mixtures (the
    shipped cases' mix_of_mix; shear-independent Ishii-Zuber): finite blocks with the
    mixture's density in the mass rows, and the chemicals restored afterwards."""
    mesh = syn.box_tet_delaunay(4, seed=2)
    mat = syn.material_for(2, 0)
    setup = syn.setup_for(3, 2)
    I, _ = syn.state_for(mesh, 2, 0)
    S = I.reshape(-1, 6)
    S[:, 0] = np.clip(S[:, 0], 7.0e7, 2.5e8)
    S[:, 4] = 1300.0
    P = I.copy()
    nd = 6
    nrp, ncol, rp, col = oracle.pattern(mesh, nd)
    v0, r0, s0, _ = oracle.assemble(mesh, mat, setup, I, P, 1e-3, rp, col)
    with oracle.magma_material(syn.magma_pair()):
        v1, r1, s1, _ = oracle.assemble(mesh, mat, setup, I, P, 1e-3, rp, col)
        pr = oracle.properties(mat, 1.0e8, 1300.0, np.array([0.5, 0.5]))
    ref, _, _ = oracle.magma_properties(syn.magma_pair(), np.array([1.0e8]), np.array([1300.0]), np.array([[0.5, 0.5]]))
    assert s0 == s1 == 0 and np.isfinite(v1).all() and np.isfinite(r1).all()
    assert not np.allclose(v1, v0)
    assert pr["rho"] == ref[0, 0] and pr["mu"] == ref[1, 0] and pr["D"] == 0.0
    v2, _, _, _ = oracle.assemble(mesh, mat, setup, I, P, 1e-3, rp, col)
    assert np.array_equal(v2, v0)


def _melt_only(oxide_wf, n_p=11):
    """A volatile-free magma: no H2O or CO2, so the mixture is the melt alone."""
    p = np.linspace(6.0e7, 3.0e8, n_p)
    m = magma.MagmaMix(name="dry", oxide_wf=oxide_wf, h2o_wf=0.0, co2_wf=0.0)
    return m.with_tables(p, np.zeros(n_p), np.zeros(n_p))


OXIDE_MM = np.array([60.084, 79.876, 101.956, 159.692, 71.846, 70.937, 40.304, 56.078, 61.979, 94.195])


def test_pin_dry_melt_density_and_heat_capacity():
    """Lange-Carmichael molar volume (chemicals.hpp:62-103, 110-120) of a dry melt,
    computed here from the oxide tables: rho = M / (V + dV/dT (T - 1673) + dV/dp (p - 1e5))."""
    wf = np.array(syn.BASALT_LIKE) / np.sum(syn.BASALT_LIKE)
    mm = OXIDE_MM * 1e-3
    M = 1.0 / np.sum(wf / mm)
    x = wf * M / mm
    V = np.sum(x * np.array([26.86, 23.16, 37.42, 42.13, 13.65, 0.0, 11.69, 16.53, 28.88, 45.07]) * 1e-6)
    dT = np.sum(x * np.array([0.0, 7.24, 0.0, 9.09, 2.92, 0.0, 3.27, 3.74, 7.68, 12.08]) * 1e-9)
    dp = np.sum(x * np.array([-1.89, -2.31, -2.26, -2.53, -0.45, 0.0, 0.27, 0.34, -2.4, -6.75]) * 1e-15)
    cp = np.sum(x * np.array([1331.0, 1392.0, 1545.0, 1434.0, 1100.0, 0.0, 2424.0, 1781.0, 1651.0, 1030.0]))
    p, T = np.array([1.0e8, 2.0e8]), np.array([1473.0, 1673.0])
    out, _, st = oracle.magma_properties([_melt_only(syn.BASALT_LIKE)], p, T, np.ones((2, 1)))
    mv = V + dT * (T - 1673.0) + dp * (p - 1e5)
    np.testing.assert_allclose(out[0], M / mv, rtol=1e-13)
    np.testing.assert_allclose(out[2], cp, rtol=1e-13)
    np.testing.assert_allclose(out[6], dT / mv, rtol=1e-12)     # alpha
    np.testing.assert_allclose(out[7], -dp / mv, rtol=1e-12)    # beta
    assert 2500.0 < out[0][0] < 2900.0


def test_pin_dry_melt_viscosity_vft():
    """Giordano et al. (2008) for a dry melt (GiordanoEtAlViscosityModel.hpp:36-116):
    log10 mu = -4.55 + B / (T - C) with B and C from the mole percents (Fe as FeO)."""
    wf = np.array(syn.TRACHYTE_LIKE, dtype=float) / np.sum(syn.TRACHYTE_LIKE)
    w = wf.copy()
    w[4] = 0.9309 * (w[3] + w[4])
    w[3] = 0.0
    w /= w.sum()
    Mv = 1.0 / np.sum(w / OXIDE_MM)
    m = 100.0 * w * Mv / OXIDE_MM
    B = (159.6 * (m[0] + m[1]) - 173.3 * m[2] + 72.1 * (m[4] + m[5]) + 75.7 * m[6] - 39.0 * m[7] - 84.1 * m[8]
         - 2.43 * (m[0] + m[1]) * (m[4] + m[5] + m[6]) - 0.91 * (m[0] + m[1] + m[2]) * (m[8] + m[9])
         + 17.6 * m[2] * (m[8] + m[9]))
    C = (2.75 * m[0] + 15.7 * (m[1] + m[2]) + 8.3 * (m[4] + m[5] + m[6]) + 10.2 * m[7] - 12.3 * (m[8] + m[9])
         + 0.3 * (m[2] + m[4] + m[5] + m[6] + m[7]) * (m[8] + m[9]))
    T = np.array([1200.0, 1400.0])
    out, _, st = oracle.magma_properties([_melt_only(syn.TRACHYTE_LIKE)], np.full(2, 1.0e8), T, np.ones((2, 1)))
    assert st == 0
    np.testing.assert_allclose(np.log10(out[1]), -4.55 + B / (T - C), rtol=1e-12)
    assert out[1][0] > out[1][1] > 1.0    # viscosity falls with temperature


# the reference project's checkout, when one is present (GALES_REFERENCE_DIR)
REF_CASE = pathlib.Path(os.environ.get("GALES_REFERENCE_DIR", "-"), "sim/fluid_mc/P0")


@pytest.mark.skipif(not (REF_CASE / "props.txt").exists(), reason="the reference's case files are not present")
def test_reads_the_reference_case_files():
    """The shipped case's own props.txt (two magma_mix blocks) and input/lookuptable
    files parse, and the mixture's properties over the tables' pressure range are finite
    and physical (format compatibility with the reference's inputs; no expected values
    ship with them)."""
    mixes = magma.read_props(REF_CASE / "props.txt")
    assert [m.name for m in mixes] == ["shoshonite", "phonolite"]
    assert all(m.gas_on_mu == "Ishii_Zuber" and m.crystal_on_mu == "none" for m in mixes)
    for m in mixes:
        magma.read_lookup_tables(REF_CASE / "input" / "lookuptable", m)
        assert len(m.p_table) == len(m.wf_l_h2o) == len(m.wf_l_co2) > 2 and m.T_table is None
    p = np.linspace(m.p_table[0] * 1.01, m.p_table[-1] * 0.99, 50)
    out, comp, st = oracle.magma_properties(mixes, p, np.full(50, 1300.0), np.full((50, 2), 0.5))
    assert st == 0 and np.isfinite(out).all()
    assert np.all((out[0] > 2000.0) & (out[0] < 3000.0)) and np.all(out[1] > 1.0)
    assert np.all(np.diff(comp[:, 3], axis=1) <= 0.0)   # less gas at higher pressure
