"""GPU parity against the CPU oracle at the benchmark workloads' own sizes.

The small cases of test_gpu_parity.py fit in one interior chunk.  These run the
production schedule: the 999,931-tet benchmark mesh (Delaunay of a jittered 54^3
lattice, 3 components, 7 dofs) compared with the oracle's full FP64 assembly
(fluid_assembly.hpp:39-68 with scatter.hpp:37-98), meshes cut into several interior
chunks (gales_asm_set_chunk) in both forms and both scatter modes with device,
page-locked and pageable buffers (the point kernel then the persistent matrix kernel per
chunk reusing one record buffer, the Morton and lowest-node-bucket element orders and
the row-prefix copies to the host), a multi-chunk hex mesh, and the adjoint on the
200k-tet workload.

Bars: CSR pattern and colouring bit-exact; FP64 form <= 1e-12 relative
(Frobenius / L2); mixed form <= 1e-6 relative, against the oracle.
"""
import os

import numpy as np
import pytest

import cases
from cases import gm, rel, syn

import autograd_harness as ah

FP64_TOL = 1e-12
MIXED_TOL = 1e-6
THREADS = os.cpu_count() or 1


def _oracle_fp64(orc, mesh, mat, setup, I, P, dt, nd):
    nrp, ncol, rp, cl = orc.pattern(mesh, nd)
    colour, nco = orc.colouring(mesh)
    vals, rhs, s, fb = orc.assemble(mesh, mat, setup, I, P, dt, rp, cl, nthreads=THREADS, colour=colour,
                                    n_colours=nco)
    assert s == 0, f"oracle status {s} at element {fb}"
    return dict(nrp=nrp, ncol=ncol, rp=rp, col=cl, colour=colour, n_colours=nco, vals=vals, rhs=rhs)


def _device_assembly(fa, I, P, dt, form):
    import torch
    dev = torch.device("cuda:0")
    lp = fa.linear_system(device=dev)
    fa.execute(torch.tensor(I, device=dev), torch.tensor(P, device=dev), dt, lp, form=form)
    torch.cuda.synchronize(dev)
    return lp.vals.cpu().numpy(), lp.rhs.cpu().numpy()


# ---------------------------------------------------------------- 999,931 tets


@pytest.fixture(scope="module")
def c1(orc, cuda_lib):
    mesh = syn.box_tet_delaunay(54, seed=1)
    mat, setup = syn.material_for(3, 0), syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, 0)
    assert mesh.n_elements == 999_931 and mesh.n_nodes == 157_464
    ref = _oracle_fp64(orc, mesh, mat, setup, I, P, 1e-3, 7)
    return mesh, mat, setup, I, P, 1e-3, ref


@pytest.mark.gpu
def test_c1_pattern_and_colouring_bit_exact(c1):
    mesh, mat, setup, I, P, dt, ref = c1
    fa = gm.FluidAssembly(mesh, mat, setup)
    row_ptr, col = fa.pattern()
    assert np.array_equal(row_ptr, ref["rp"]) and np.array_equal(col, ref["col"])
    g_rp, g_col = fa.node_graph()
    assert np.array_equal(g_rp, ref["nrp"]) and np.array_equal(g_col, ref["ncol"])
    colour, nco = fa.colouring()
    assert nco == ref["n_colours"] and np.array_equal(colour, ref["colour"])


@pytest.mark.gpu
@pytest.mark.parametrize("scatter", ["atomic", "coloured"])
def test_c1_fp64_within_1e12_of_oracle(scatter, c1):
    mesh, mat, setup, I, P, dt, ref = c1
    fa = gm.FluidAssembly(mesh, mat, setup)
    if scatter == "coloured":
        fa.set_scatter(gm.SCATTER_COLOURED)
    v, b = _device_assembly(fa, I, P, dt, gm.FORM_FP64)
    assert rel(v, ref["vals"]) <= FP64_TOL
    assert rel(b, ref["rhs"]) <= FP64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("scatter", ["atomic", "coloured"])
def test_c1_mixed_within_1e6_of_oracle(scatter, c1):
    mesh, mat, setup, I, P, dt, ref = c1
    fa = gm.FluidAssembly(mesh, mat, setup)
    if scatter == "coloured":
        fa.set_scatter(gm.SCATTER_COLOURED)
    v, b = _device_assembly(fa, I, P, dt, gm.FORM_MIXED)
    assert rel(v, ref["vals"]) <= MIXED_TOL
    assert rel(b, ref["rhs"]) <= MIXED_TOL


# ------------------------------------------------- several interior chunks, all buffers


@pytest.fixture(scope="module")
def chunked(orc, cuda_lib):
    mesh = syn.box_tet_delaunay(25, seed=2)
    mat, setup = syn.material_for(3, 1), syn.setup_for(3, 3)
    I, P = syn.state_for(mesh, 3, 1)
    ref = _oracle_fp64(orc, mesh, mat, setup, I, P, 1e-3, 7)
    return mesh, mat, setup, I, P, 1e-3, ref


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed"])
@pytest.mark.parametrize("scatter", ["atomic", "coloured"])
@pytest.mark.parametrize("buffers", ["device", "pinned", "pageable"])
def test_multichunk_tets_match_oracle(form, scatter, buffers, chunked):
    import torch
    mesh, mat, setup, I, P, dt, ref = chunked
    f = gm.FORM_MIXED if form == "mixed" else gm.FORM_FP64
    tol = MIXED_TOL if form == "mixed" else FP64_TOL
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_chunk(14_592)
    if scatter == "coloured":
        fa.set_scatter(gm.SCATTER_COLOURED)
    dev = torch.device("cuda:0")
    if buffers == "device":
        lp = fa.linear_system(device=dev)
        Iin, Pin = torch.tensor(I, device=dev), torch.tensor(P, device=dev)
    elif buffers == "pinned":
        lp = gm.LinearSystem(ref["rp"], ref["col"], torch.zeros(len(ref["vals"]), dtype=torch.float64).pin_memory(),
                             torch.zeros(len(ref["rhs"]), dtype=torch.float64).pin_memory())
        Iin, Pin = torch.from_numpy(I).pin_memory(), torch.from_numpy(P).pin_memory()
    else:
        lp = fa.linear_system()
        Iin, Pin = I, P
    n0 = fa.launch_count()
    for _ in range(2):      # a second call reuses the record buffer, the copy events and the orders
        fa.execute(Iin, Pin, dt, lp, form=f)
        torch.cuda.synchronize(dev)
        v = lp.vals.cpu().numpy() if torch.is_tensor(lp.vals) else lp.vals
        b = lp.rhs.cpu().numpy() if torch.is_tensor(lp.rhs) else lp.rhs
        assert rel(v, ref["vals"]) <= tol
        assert rel(b, ref["rhs"]) <= tol
    # the mesh spans at least five interior chunks: a point and a matrix launch each
    assert (fa.launch_count() - n0) // 2 >= 2 * 5
    assert mesh.n_elements >= 5 * 14_592


# ------------------------------------------------------------- hexes, several chunks


@pytest.fixture(scope="module")
def hexes(orc, cuda_lib):
    mesh = syn.box_hex(32, 32, 24, jitter=0.1, seed=4)
    mat, setup = syn.material_for(4, 0), syn.setup_for(3, 4)
    I, P = syn.state_for(mesh, 4, 0)
    ref = _oracle_fp64(orc, mesh, mat, setup, I, P, 1e-3, 8)
    return mesh, mat, setup, I, P, 1e-3, ref


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_multichunk_hexes_match_oracle(form, hexes):
    mesh, mat, setup, I, P, dt, ref = hexes
    assert mesh.n_elements >= 3 * 7_296
    fa = gm.FluidAssembly(mesh, mat, setup)
    fa.set_chunk(7_296)                          # several chunks
    v, b = _device_assembly(fa, I, P, dt, gm.FORM_MIXED if form == "mixed" else gm.FORM_FP64)
    tol = MIXED_TOL if form == "mixed" else FP64_TOL
    assert rel(v, ref["vals"]) <= tol
    assert rel(b, ref["rhs"]) <= tol


# ------------------------------------------------------------- adjoint, 200k tets


@pytest.fixture(scope="module")
def c3(cuda_lib):
    mesh = syn.box_tet_delaunay(32, seed=3)
    mat = syn.material_for(3, 0)
    mat = ah.material_from_theta(mat, ah.theta_of(mat))
    setup = syn.setup_for(3, 3)
    # nonzero wall velocity: compute_h's rank-one branch is decided by rounding noise
    I, P = syn.state_for(mesh, 3, 0, perturb=1e-4, no_slip_flag=-1)
    assert mesh.n_elements >= 199_000
    return mesh, mat, setup, I, P, 1e-3


@pytest.mark.gpu
def test_c3_frozen_vjp_is_oracle_transpose(c3, orc):
    import scipy.sparse as sp
    mesh, mat, setup, I, P, dt = c3
    ref = _oracle_fp64(orc, mesh, mat, setup, I, P, dt, 7)
    A = sp.csr_matrix((ref["vals"], ref["col"], ref["rp"]), shape=(len(ref["rhs"]),) * 2)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lam = np.random.default_rng(1).normal(size=fa.n_rows)
    lam /= np.linalg.norm(lam)
    g = np.zeros(fa.n_rows)
    fa.vjp(I, P, dt, lam, gm.VJP_FROZEN, g)
    assert rel(g, A.T @ lam) <= 1e-12


def _lb(fa, I, P, dt, lam):
    b = np.zeros(fa.n_rows)
    fa.residual(I, P, dt, b, form=gm.FORM_FP64)
    return float(lam @ b), float(np.abs(lam * b).sum())


@pytest.mark.gpu
def test_c3_exact_vjp_matches_central_differences(c3):
    mesh, mat, setup, I, P, dt = c3
    fa = gm.FluidAssembly(mesh, mat, setup)
    rng = np.random.default_rng(11)
    lam = rng.normal(size=fa.n_rows)
    lam /= np.linalg.norm(lam)
    g = np.zeros(fa.n_rows)
    th = np.zeros(9)
    fa.vjp(I, P, dt, lam, gm.VJP_EXACT, g, th)
    scale = np.abs(I.reshape(-1, fa.nd)).max(axis=0)
    # three state directions, fourth-order central differences (on 200k elements the
    # second-order truncation error of a 1e-6 step is ~1e-2, of 1e-7 ~1e-4); a shorter
    # step stands in where a kink of the residual (min() in tau's caps, |.| in the dc
    # length) lies within the step
    for k in range(3):
        d = (rng.normal(size=I.shape).reshape(-1, fa.nd) * scale).ravel()
        an = float(g @ d)
        res = []
        for h in (1e-6, 1e-7):
            f = [_lb(fa, I + m * h * d, P, dt, lam) for m in (1, -1, 2, -2)]
            fd = (8 * (f[0][0] - f[1][0]) - (f[2][0] - f[3][0])) / (12 * h)
            noise = 10 * 2.2e-16 * max(x[1] for x in f) / h
            res.append((abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + noise, h, fd))
        assert any(r[0] for r in res), (k, an, res)
    # one direction in the 9 material parameters (3 densities, 3 viscosities, 3 heat
    # capacities), fourth-order differences.  A parameter step moves every point's tau
    # caps (min()) at once, and with lambda spread over all 800k points thousands of
    # them cross a kink within any step, which bounds the difference quotient's accuracy
    # near 1e-3; lambda is therefore supported on the rows of one corner of the box
    # (about a thousand elements), while the VJP still runs over the whole mesh.
    corner = np.all(mesh.coords < 0.18, axis=1)
    lam = (lam.reshape(-1, fa.nd) * corner[:, None]).ravel()
    lam /= np.linalg.norm(lam)
    g = np.zeros(fa.n_rows)
    th = np.zeros(9)
    fa.vjp(I, P, dt, lam, gm.VJP_EXACT, g, th)
    theta = ah.theta_of(mat)
    v = rng.normal(size=9)
    an = float((th * theta) @ v)
    _, L_abs = _lb(fa, I, P, dt, lam)
    ok = []
    for h in (1e-3, 1e-4, 1e-5):
        vals = []
        for m in (1, -1, 2, -2):
            f2 = gm.FluidAssembly(mesh, ah.material_from_theta(mat, theta * (1 + m * h * v)), setup)
            vals.append(_lb(f2, I, P, dt, lam)[0])
            f2.close()
        fd = (8 * (vals[0] - vals[1]) - (vals[2] - vals[3])) / (12 * h)
        ok.append((abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + 10 * 2.2e-16 * L_abs / h, h, fd))
    assert any(o[0] for o in ok), (an, ok)
