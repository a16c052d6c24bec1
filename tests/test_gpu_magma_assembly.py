"""The assembly with magma mixtures as its material (the shipped cases' props.txt
mix_of_mix of magma_mix, fluid_properties.hpp:171-200), against the oracle's assembly
with the same magmas (gor_set_magma).

The point properties are the magma mixture at P with shear rate 0 and at I (and at the
boundary points) with the point's shear rate (fluid_2d.hpp:186, 193-194, 234-235;
compute_shear_rate, non_newtonian.hpp:23-39), which the shear-dependent crystal model
(Caricchi 2007) reads.  Bars as for the chemicals: FP64 form <= 1e-12, mixed <= 1e-6
relative; the differences come from the CUDA and host math libraries (pow, log, exp,
erf, tanh in the magma model).  The adaptive time step, the nodal secondary variables and
the gas fractions of secondary_dofs (pp_vf_g) run with the same magmas.
"""
import numpy as np
import pytest

import cases
from cases import gm, rel, syn

MODELS = [("Ishii_Zuber", "none", 0.0, 0), ("none", "Caricchi", 0.3, 0), ("Ishii_Zuber", "Einstein_Roscoe", 0.1, 7)]


def _magma_state(mesh, nc, seed=0, perturb=1e-4):
    """state_for's fields with the pressure mapped into the solubility tables' range
    (75..275 MPa) and T in 1223..1323 K."""
    I, P = syn.state_for(mesh, nc, seed, perturb=0.0)
    nd = gm.nb_dofs(mesh.dim, nc)
    S = I.reshape(-1, nd)
    S[:, 0] = 7.5e7 + 2.0e8 * (S[:, 0] - S[:, 0].min()) / (S[:, 0].max() - S[:, 0].min())
    I = S.ravel().copy()
    rng = np.random.default_rng(seed + 7)
    scale = np.abs(S).max(axis=0)
    P = (S + perturb * rng.normal(size=S.shape) * scale).ravel()
    return I, P


def _case(kind, gas, crystal, cf, n_T):
    mesh = {"tri": lambda: syn.channel_tri(16, 8), "quad": lambda: syn.channel_quad(12, 6, jitter=0.2, seed=0),
            "tet": lambda: syn.box_tet_delaunay(6, seed=1), "hex": lambda: syn.box_hex(4, 4, 3, jitter=0.1, seed=2)}[kind]()
    comps = syn.magma_pair(gas_on_mu=gas, crystal_on_mu=crystal, crystal_fraction=cf, n_T=n_T)
    mat = syn.material_for(2, 0)          # the chemicals the magmas replace
    setup = syn.setup_for(mesh.dim, 2, dirichlet_T_everywhere=True)
    I, P = _magma_state(mesh, 2)
    return mesh, comps, mat, setup, I, P, 1e-3


def _oracle(orc, mesh, comps, mat, setup, I, P, dt, nd):
    nrp, ncol, rp, col = orc.pattern(mesh, nd)
    with orc.magma_material(comps):
        vals, rhs, s, fb = orc.assemble(mesh, mat, setup, I, P, dt, rp, col)
    assert s == 0, (s, fb)
    return vals, rhs


@pytest.mark.gpu
@pytest.mark.parametrize("gas,crystal,cf,n_T", MODELS)
@pytest.mark.parametrize("kind", ["tri", "quad", "tet", "hex"])
def test_magma_assembly_matches_oracle(kind, gas, crystal, cf, n_T, cuda_lib, orc):
    magma = pytest.importorskip("gales-multi-fluid_gb300.magma")
    mesh, comps, mat, setup, I, P, dt = _case(kind, gas, crystal, cf, n_T)
    mm = magma.MagmaMaterial(comps)
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_magma(mm)
    vals, rhs = _oracle(orc, mesh, comps, mat, setup, I, P, dt, fa.nd)
    for form, tol in ((gm.FORM_FP64, 1e-12), (gm.FORM_MIXED, 1e-6)):
        lp = fa.linear_system()
        fa.execute(I, P, dt, lp, form=form)
        assert rel(lp.vals, vals) <= tol, (form, rel(lp.vals, vals))
        assert rel(lp.rhs, rhs) <= tol, (form, rel(lp.rhs, rhs))
    # detached: the chemicals' assembly again
    fa.set_magma(None)
    lp = fa.linear_system()
    fa.execute(I, P, dt, lp, form=gm.FORM_FP64)
    nrp, ncol, rp, col = orc.pattern(mesh, fa.nd)
    v0, r0, s0, _ = orc.assemble(mesh, mat, setup, I, P, dt, rp, col)
    assert rel(lp.vals, v0) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("scatter", ["atomic", "coloured"])
def test_magma_multichunk_and_scatter_modes(scatter, cuda_lib, orc):
    """A mesh of several interior chunks, both scatter modes, device buffers."""
    import torch
    magma = pytest.importorskip("gales-multi-fluid_gb300.magma")
    mesh = syn.box_tet_delaunay(16, seed=5)
    comps = syn.magma_pair(crystal_on_mu="Caricchi", crystal_fraction=0.2)
    mat, setup = syn.material_for(2, 0), syn.setup_for(3, 2)
    I, P = _magma_state(mesh, 2, seed=3)
    mm = magma.MagmaMaterial(comps)
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_magma(mm)
    fa.set_chunk(4096)                      # several interior chunks
    assert mesh.n_elements >= 3 * 4096
    if scatter == "coloured":
        fa.set_scatter(gm.SCATTER_COLOURED)
    vals, rhs = _oracle(orc, mesh, comps, mat, setup, I, P, 1e-3, fa.nd)
    dev = torch.device("cuda:0")
    for form, tol in ((gm.FORM_FP64, 1e-12), (gm.FORM_MIXED, 1e-6)):
        lp = fa.linear_system(device=dev)
        fa.execute(torch.tensor(I, device=dev), torch.tensor(P, device=dev), 1e-3, lp, form=form)
        assert rel(lp.vals.cpu().numpy(), vals) <= tol
        assert rel(lp.rhs.cpu().numpy(), rhs) <= tol


@pytest.mark.gpu
def test_magma_frozen_vjp_and_exact_unsupported(cuda_lib):
    magma = pytest.importorskip("gales-multi-fluid_gb300.magma")
    mesh, comps, mat, setup, I, P, dt = _case("tet", "Ishii_Zuber", "none", 0.0, 0)
    mm = magma.MagmaMaterial(comps)
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_magma(mm)
    lp = fa.linear_system()
    fa.execute(I, P, dt, lp, form=gm.FORM_FP64)
    lam = np.random.default_rng(2).normal(size=fa.n_rows)
    g = np.zeros(fa.n_rows)
    fa.vjp(I, P, dt, lam, gm.VJP_FROZEN, g)
    assert rel(g, lp.matrix_scipy().T @ lam) <= 1e-12
    with pytest.raises(gm.GalesError) as e:
        fa.vjp(I, P, dt, lam, gm.VJP_EXACT, g, np.zeros(6))
    assert e.value.code == gm.abi.ERR_UNSUPPORTED


@pytest.mark.gpu
def test_magma_out_of_table_state_is_reported(cuda_lib):
    magma = pytest.importorskip("gales-multi-fluid_gb300.magma")
    mesh, comps, mat, setup, I, P, dt = _case("tri", "Ishii_Zuber", "none", 0.0, 0)
    mm = magma.MagmaMaterial(comps)
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_magma(mm)
    I2 = I.copy()
    I2.reshape(-1, fa.nd)[5, 0] = 1.0e6          # below the tables (60 MPa): the reference stops
    lp = fa.linear_system()
    with pytest.raises(gm.GalesError) as e:
        fa.execute(I2, P, dt, lp, form=gm.FORM_FP64)
    assert e.value.code & gm.abi.ERR_MAGMA
    fa.execute(I, P, dt, lp, form=gm.FORM_FP64)   # the handle stays usable


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["tri", "tet"])
def test_magma_adaptive_dt_secondary_dofs_and_fractions(kind, cuda_lib, orc):
    magma = pytest.importorskip("gales-multi-fluid_gb300.magma")
    mesh, comps, mat, setup, I, P, dt = _case(kind, "Ishii_Zuber", "Einstein_Roscoe", 0.1, 0)
    mm = magma.MagmaMaterial(comps)
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_magma(mm)
    nd, dim = fa.nd, mesh.dim
    S = I.reshape(-1, nd)
    Y = np.stack([S[:, dim + 2], 1.0 - S[:, dim + 2]], axis=1)
    d_el = np.zeros(mesh.n_elements)
    fa.adaptive_dt(I, dt, 0.5, 1e-9, 1.0, dt_el=d_el)
    with orc.magma_material(comps):
        ref_dt = orc.adaptive_dt(mesh, mat, setup, I, dt, 0.5)
        props = [orc.properties(mat, S[i, 0], S[i, dim + 1], Y[i]) for i in range(len(S))]
        fr = orc.magma_fractions(S[:, 0], S[:, dim + 1], Y)
    assert rel(d_el, ref_dt) <= 1e-12
    sec = fa.secondary_dofs(I)
    keys = ["rho", "mu", "cp", "cv", "alpha", "beta", "kappa", "c"]
    ref = np.array([[pr[k] for pr in props] for k in keys])
    for f in range(8):
        assert rel(sec[f], ref[f]) <= 1e-12, keys[f]
    got = fa.magma_fractions(I)
    assert got.shape == (2 * 2 + 6, mesh.n_nodes)
    for f in range(got.shape[0]):
        assert rel(got[f], fr[f]) <= 1e-12, f
    assert np.all(got[-6] > 0.0)                 # some gas at these pressures


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["magma+custom", "magma+gas", "custom+chemical", "three"])
@pytest.mark.parametrize("elem", ["tri", "tet"])
def test_submixture_kinds_assembly_matches_oracle(kind, elem, cuda_lib, orc):
    """custom_mix and ch_as_mix sub-mixtures beside magma_mix (fluid_properties_reader.hpp:
    127-141, mixtures.hpp:25-101) in the assembly, both forms, against the oracle."""
    import test_magma as tm
    magma = pytest.importorskip("gales-multi-fluid_gb300.magma")
    comps = tm._with_submixtures(kind)
    nc = len(comps)
    mesh = syn.channel_tri(16, 8) if elem == "tri" else syn.box_tet_delaunay(6, seed=1)
    mat = syn.material_for(nc, 0)
    setup = syn.setup_for(mesh.dim, nc)
    I, P = _magma_state(mesh, nc)
    mm = magma.MagmaMaterial(comps)
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_magma(mm)
    vals, rhs = _oracle(orc, mesh, comps, mat, setup, I, P, 1e-3, fa.nd)
    for form, tol in ((gm.FORM_FP64, 1e-12), (gm.FORM_MIXED, 1e-6)):
        lp = fa.linear_system()
        fa.execute(I, P, 1e-3, lp, form=form)
        assert rel(lp.vals, vals) <= tol, (form, rel(lp.vals, vals))
        assert rel(lp.rhs, rhs) <= tol, (form, rel(lp.rhs, rhs))
