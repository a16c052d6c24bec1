"""GPU parity: the CUDA assembly against the CPU oracle on identical meshes and states.

Bars (from the hot-path contract):
  - CSR pattern and element colouring: bit-exact
  - FP64 form: relative Frobenius (matrix) and L2 (rhs) error <= 1e-12
  - mixed form: relative error <= 1e-6 against the FP64 oracle
"""
import numpy as np
import pytest

import cases
from cases import rel

FP64_TOL = 1e-12
MIXED_TOL = 1e-6

KINDS = [("tri", 2), ("tri", 1), ("tri", 3), ("tri", 4), ("quad", 2), ("quad", 3), ("tet", 3), ("tet", 1),
         ("tet", 2), ("hex", 4), ("hex", 2)]


def _run(gm, orc, mesh, mat, setup, I, P, dt, form):
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system()
    fa.execute(I, P, dt, lp, form=form)
    ref_vals, ref_rhs, s, fb = orc.assemble(mesh, mat, setup, I, P, dt, lp.row_ptr, lp.col)
    assert s == 0, f"oracle status {s} at {fb}"
    return fa, lp, ref_vals, ref_rhs


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", KINDS)
def test_pattern_and_colouring_bit_exact(kind, nc, cuda_lib, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    nd = gm.nb_dofs(mesh.dim, nc)
    row_ptr, col = fa.pattern()
    nrp, ncol, rp, cl = orc.pattern(mesh, nd)
    assert np.array_equal(row_ptr, rp)
    assert np.array_equal(col, cl)
    g_rp, g_col = fa.node_graph()
    assert np.array_equal(g_rp, nrp) and np.array_equal(g_col, ncol)
    colour, ncolours = fa.colouring()
    ocol, onc = orc.colouring(mesh)
    assert ncolours == onc and np.array_equal(colour, ocol)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", KINDS)
def test_fp64_matches_oracle(kind, nc, cuda_lib, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_FP64)
    assert rel(lp.vals, vals) <= FP64_TOL
    assert rel(lp.rhs, rhs) <= FP64_TOL


@pytest.mark.gpu
def test_fp64_channel_c0(cuda_lib, gm, orc):
    """The 2D channel workload (64 x 32 quads -> 4096 triangles, 2145 nodes, 5 dofs)."""
    mesh, mat, setup, I, P, dt = cases.make("tri_c0", 2)
    assert mesh.n_elements == 4096 and mesh.n_nodes == 2145
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_FP64)
    assert rel(lp.vals, vals) <= FP64_TOL
    assert rel(lp.rhs, rhs) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", [("tri", 2), ("quad", 2), ("tet", 3), ("hex", 4)])
def test_mixed_within_1e6(kind, nc, cuda_lib, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_MIXED)
    assert rel(lp.vals, vals) <= MIXED_TOL
    assert rel(lp.rhs, rhs) <= MIXED_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [2019, 2001, 2007, 2014, 0])
@pytest.mark.parametrize("kind", ["tri", "tet"])
def test_tau_variants(variant, kind, cuda_lib, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make(kind, 3, setup_kw=dict(tau=variant))
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_FP64)
    assert rel(lp.vals, vals) <= FP64_TOL
    assert rel(lp.rhs, rhs) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [2001, 2007, 2014, 0])
@pytest.mark.parametrize("kind", ["tri", "tet", "hex"])
def test_mixed_tau_variants(variant, kind, cuda_lib, gm, orc):
    nc = 4 if kind == "hex" else 3
    mesh, mat, setup, I, P, dt = cases.make(kind, nc, setup_kw=dict(tau=variant))
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_MIXED)
    assert rel(lp.vals, vals) <= MIXED_TOL
    assert rel(lp.rhs, rhs) <= MIXED_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("sharp", [1.0, 1.5, 2.0])
@pytest.mark.parametrize("steady", [False, True])
def test_dc_and_steady(sharp, steady, cuda_lib, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make("tri", 2, setup_kw=dict(dc_sharp=sharp, steady_state=steady,
                                                                     dc_scale_fact=0.7))
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_FP64)
    assert rel(lp.vals, vals) <= FP64_TOL
    assert rel(lp.rhs, rhs) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", [("tri", 3), ("quad", 2), ("tet", 3), ("hex", 2)])
def test_boundary_overrides(kind, nc, cuda_lib, gm, orc):
    """Neumann stress/heat/species overrides and prescribed mass flux on side flags,
    T Dirichlet on every node (the shipped P0 policy)."""
    mesh, mat, setup, I, P, dt = cases.make(kind, nc, T_everywhere=True)
    dim = mesh.dim
    open_flag = 2
    setup.neumann_tau(open_flag, 0, 0, 3.0e3).neumann_tau(open_flag, 0, dim - 1, -1.5e3)
    setup.neumann_q(open_flag, dim - 1, 12.0)
    if nc > 1:
        setup.neumann_J(open_flag, 0, 0, 1e-3)
    setup.mass_flux(open_flag, dim - 1, 0.37)
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, P, dt, gm.FORM_FP64)
    assert rel(lp.vals, vals) <= FP64_TOL
    assert rel(lp.rhs, rhs) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", [("tri", 2), ("tet", 3), ("hex", 4)])
def test_coloured_scatter_equals_atomic(kind, nc, cuda_lib, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp_a = fa.linear_system()
    fa.execute(I, P, dt, lp_a)
    fa.set_scatter(gm.SCATTER_COLOURED)
    lp_c = fa.linear_system()
    fa.execute(I, P, dt, lp_c)
    assert rel(lp_c.vals, lp_a.vals) <= 1e-14
    assert rel(lp_c.rhs, lp_a.rhs) <= 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_residual_only_equals_assembled_rhs(form, cuda_lib, gm):
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system()
    fa.execute(I, P, dt, lp, form=form)
    rhs = np.zeros(fa.n_rows)
    fa.residual(I, P, dt, rhs, form=form)
    assert rel(rhs, lp.rhs) <= 1e-14


@pytest.mark.gpu
def test_device_pointers_and_stream(cuda_lib, gm):
    import torch
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp_h = fa.linear_system()
    fa.execute(I, P, dt, lp_h)
    lp_d = fa.linear_system(device="cuda")
    Id = torch.from_numpy(I).cuda()
    Pd = torch.from_numpy(P).cuda()
    s = torch.cuda.Stream()
    fa.execute(Id, Pd, dt, lp_d, stream=s.cuda_stream)
    assert rel(lp_d.vals.cpu().numpy(), lp_h.vals) <= 1e-14
    assert rel(lp_d.rhs.cpu().numpy(), lp_h.rhs) <= 1e-14


@pytest.mark.gpu
def test_p_equals_i_newton_iteration0(cuda_lib, gm, orc):
    """At Newton iteration 0 the predictor sets P := I (fluid_updater.hpp:18-21)."""
    mesh, mat, setup, I, P, dt = cases.make("tet", 3, perturb=0.0)
    fa, lp, vals, rhs = _run(gm, orc, mesh, mat, setup, I, I.copy(), dt, gm.FORM_FP64)
    assert rel(lp.vals, vals) <= FP64_TOL
    assert rel(lp.rhs, rhs) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed"])
@pytest.mark.parametrize("offset", [0, 1])
@pytest.mark.parametrize("chunks", ["one", "several"])
@pytest.mark.parametrize("kind,nc", [("tet", 3), ("hex", 4)])
def test_outputs_cleared_by_the_call(kind, nc, chunks, offset, form, cuda_lib, gm, orc):
    """The call clears A and b itself (with the atomic scatter and one interior chunk,
    inside the point launch; over several chunks with a clear kernel): outputs
    prefilled with NaN, at a 16-byte-aligned and at an odd-word offset, give the
    oracle's values, twice in a row, and the words beside them stay untouched."""
    import torch
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    if chunks == "several":
        chunk = max(4, mesh.n_elements // 5 // 4 * 4)
        fa.set_chunk(chunk)
        assert mesh.n_elements > 3 * chunk
    row_ptr, col = fa.pattern()
    nnz, nr = int(row_ptr[-1]), len(row_ptr) - 1
    dev = torch.device("cuda:0")
    vbuf = torch.full((nnz + 2,), float("nan"), dtype=torch.float64, device=dev)
    rbuf = torch.full((nr + 2,), float("nan"), dtype=torch.float64, device=dev)
    lp = gm.LinearSystem(row_ptr, col, vbuf[offset:offset + nnz], rbuf[offset:offset + nr])
    f = gm.FORM_MIXED if form == "mixed" else gm.FORM_FP64
    tol = MIXED_TOL if form == "mixed" else FP64_TOL
    Id, Pd = torch.tensor(I, device=dev), torch.tensor(P, device=dev)
    ref_vals, ref_rhs, s, fb = orc.assemble(mesh, mat, setup, I, P, dt, row_ptr, col)
    assert s == 0
    for _ in range(2):
        fa.execute(Id, Pd, dt, lp, form=f)
        torch.cuda.synchronize(dev)
        assert rel(lp.vals.cpu().numpy(), ref_vals) <= tol
        assert rel(lp.rhs.cpu().numpy(), ref_rhs) <= tol
    outside_v = [i for i in range(nnz + 2) if not offset <= i < offset + nnz]
    outside_r = [i for i in range(nr + 2) if not offset <= i < offset + nr]
    assert bool(torch.isnan(vbuf[outside_v]).all()) and bool(torch.isnan(rbuf[outside_r]).all())
