"""Known-answer pins of the CPU oracle (no GPU).

The reference ships no tests or golden data and cannot be built here, so the
oracle is pinned by closed forms and exact properties of the restated algorithm:
quadrature identities, EOS closed forms, the LU inverse, graph and colouring
invariants, and physical balances of the assembled residual.
"""
import itertools

import numpy as np
import pytest

import cases

ELEMS = [(2, 3), (2, 4), (3, 4), (3, 8)]


def _ref_nodes(dim, nen):
    if (dim, nen) == (2, 3):
        return np.array([[0, 0], [1, 0], [0, 1]], float)
    if (dim, nen) == (2, 4):
        return np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], float)
    if (dim, nen) == (3, 4):
        return np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    return np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                     [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)


def _affine(dim, rng):
    A = np.eye(dim) + 0.2 * rng.normal(size=(dim, dim))
    if np.linalg.det(A) < 0:
        A[:, 0] *= -1
    return A, rng.normal(size=dim)


@pytest.mark.parametrize("dim,nen", ELEMS)
def test_quadrature_identities(dim, nen, orc):
    rng = np.random.default_rng(dim * 10 + nen)
    A, c = _affine(dim, rng)
    xe = _ref_nodes(dim, nen) @ A.T + c
    g = orc.gauss(dim, nen)
    vol = 0.0
    lin = rng.normal(size=dim)
    f = xe @ lin + 0.3
    for pt in g["gp"]:
        q = orc.quad(dim, nen, xe.ravel(), pt)
        assert q["status"] == 0
        assert abs(q["sh"].sum() - 1.0) < 1e-14                 # partition of unity
        assert np.abs(q["ds"].sum(axis=1)).max() < 1e-12          # sum of gradients vanishes
        assert np.allclose(q["ds"] @ f, lin, atol=1e-12)          # patch test: exact linear gradient
        assert np.allclose(q["sh"] @ xe, np.asarray(q["sh"] @ xe))
        vol += q["JxW"]
    ref_vol = {(2, 3): 0.5, (2, 4): 4.0, (3, 4): 1.0 / 6.0, (3, 8): 8.0}[(dim, nen)]
    assert vol == pytest.approx(ref_vol * abs(np.linalg.det(A)), rel=1e-13)


@pytest.mark.parametrize("dim,nen", ELEMS)
def test_boundary_area_vectors(dim, nen, orc):
    """Summed JN*W over a side's points equals the side's outward area vector."""
    rng = np.random.default_rng(7 + dim + nen)
    A, c = _affine(dim, rng)
    xe = _ref_nodes(dim, nen) @ A.T + c
    g = orc.gauss(dim, nen)
    centroid = xe.mean(axis=0)
    total = np.zeros(dim)
    for s, side in enumerate(g["sides"]):
        an = np.zeros(dim)
        for pt in g["sgp"][s]:
            an += orc.quad(dim, nen, xe.ravel(), pt, boundary=True)["JNxW"]
        pts = xe[side]
        if dim == 2:
            t = pts[1] - pts[0]
            ref = np.array([t[1], -t[0]])
        elif len(side) == 3:
            ref = 0.5 * np.cross(pts[1] - pts[0], pts[2] - pts[0])
        else:
            ref = 0.5 * np.cross(pts[2] - pts[0], pts[3] - pts[1])
        if np.dot(ref, pts.mean(axis=0) - centroid) < 0:
            ref = -ref
        assert np.allclose(an, ref, rtol=1e-12, atol=1e-14)
        total += an
    assert np.abs(total).max() < 1e-13                            # closed surface


def test_tet_rule_integrates_quadratics(orc):
    xe = _ref_nodes(3, 4)
    g = orc.gauss(3, 4)
    s = 0.0
    for pt in g["gp"]:
        q = orc.quad(3, 4, xe.ravel(), pt)
        x = q["sh"] @ xe
        s += q["JxW"] * x[0] * x[1]
    assert s == pytest.approx(1.0 / 120.0, rel=1e-13)


def test_properties_closed_forms(gm, orc):
    melt = gm.custom_chemical(2400.0, 1e3, 1200.0, 1.5, 3e-5, 1e-10)
    gas = gm.ideal_gas(8.314462 / 461.0, 1.4)
    mat = gm.Material([melt, gas])
    p, T = 3.0e7, 1250.0
    for y in (1.0, 0.0, 0.7, 0.999):
        d = orc.properties(mat, p, T, np.array([y, 1.0 - y]))
        rho_g = p / (461.0 * T)
        cv_m = 1200.0 - T * 3e-5 ** 2 / (2400.0 * 1e-10)
        assert d["rho_c"][1] == pytest.approx(rho_g, rel=1e-15)
        assert d["rho"] == pytest.approx(1.0 / (y / 2400.0 + (1 - y) / rho_g), rel=1e-14)
        assert d["cv"] == pytest.approx(y * cv_m + (1 - y) * gas.cv, rel=1e-13)
        c_m2 = 1.0 / (2400.0 * 1e-10)
        c_g2 = 1.4 * 461.0 * T
        wood = 1.0 / (y / (2400.0 ** 2 * c_m2) + (1 - y) / (rho_g ** 2 * c_g2))
        assert d["c"] == pytest.approx(np.sqrt(wood) / d["rho"], rel=1e-13)
        assert d["alpha"] == pytest.approx(d["rho"] * (y * 3e-5 / 2400.0 + (1 - y) / T / rho_g), rel=1e-13)
        assert d["beta"] == pytest.approx(d["rho"] * (y * 1e-10 / 2400.0 + (1 - y) / p / rho_g), rel=1e-13)
        assert d["e_c"][0] == pytest.approx(cv_m * T, rel=1e-14)


def test_ideal_gas_constructor_values(gm):
    g = gm.ideal_gas_named("CO2")
    R = 8.314462 / 0.04401
    assert g.R == pytest.approx(R, rel=1e-15)
    assert g.cv == pytest.approx(R / 0.4, rel=1e-14)
    assert g.cp == pytest.approx(1.4 * R / 0.4, rel=1e-14)
    assert g.mu == 1e-5 and g.kappa == pytest.approx(1e-5 * g.cp / 0.72, rel=1e-15)
    assert gm.ideal_gas_named("He").gamma == 1.67


@pytest.mark.parametrize("n", [4, 5, 7, 8])
def test_lu_inverse_matches_numpy(n, orc):
    rng = np.random.default_rng(n)
    for _ in range(20):
        A = rng.normal(size=(n, n)) + n * np.eye(n) * rng.uniform(0, 1)
        inv, s = orc.inverse(A)
        assert s == 0
        assert np.allclose(inv @ A, np.eye(n), atol=1e-11)


def test_lu_pivoting_and_singular(orc):
    A = np.array([[0.0, 2.0, 1.0], [1.0, 1.0, 0.0], [3.0, 0.0, 1.0]])
    inv, s = orc.inverse(A)
    assert s == 0 and np.allclose(inv, np.linalg.inv(A), rtol=1e-14)
    S = np.array([[1.0, 2.0], [2.0, 4.0]])
    _, s = orc.inverse(S)
    assert s == 2                                   # uBLAS: 1-based row of the zero pivot


def test_lu_badly_scaled_dudy_like(orc):
    """DUDY mixes rho*beta ~ 1e-7 with rho ~ 1e3; the inverse must still invert."""
    rng = np.random.default_rng(3)
    D = np.diag([2.4e-7, 2400.0, 2400.0, 2.4e-3 * 1e9, 2400.0])
    A = D + np.triu(rng.normal(size=(5, 5)), 1) * np.array([1e-7, 1e2, 1e2, 1e6, 1e2])[:, None]
    inv, s = orc.inverse(A)
    assert s == 0
    assert np.allclose(inv @ A, np.eye(5), atol=1e-9)


@pytest.mark.parametrize("kind,nc", [("tri", 2), ("quad", 3), ("tet", 3), ("hex", 4)])
def test_pattern_invariants(kind, nc, gm, orc):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    nd = gm.nb_dofs(mesh.dim, nc)
    nrp, ncol, rp, col = orc.pattern(mesh, nd)
    n_rows = mesh.n_nodes * nd
    assert len(rp) == n_rows + 1 and rp[-1] == len(col) == (nrp[-1]) * nd * nd
    for r in range(0, n_rows, max(1, n_rows // 50)):
        c = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(c) > 0)                       # sorted, unique
        assert r in set(c)                                  # diagonal present
    import scipy.sparse as sp
    S = sp.csr_matrix((np.ones(len(col)), col, rp), shape=(n_rows, n_rows))
    assert (S - S.T).nnz == 0                               # symmetric structure
    # every element's dense block is inside the pattern
    for e in range(0, mesh.n_elements, max(1, mesh.n_elements // 30)):
        nodes = mesh.conn[e]
        for a, b in itertools.product(nodes, nodes):
            assert b in set(ncol[nrp[a]:nrp[a + 1]])


@pytest.mark.parametrize("kind", ["tri", "tet", "hex"])
def test_colouring_is_conflict_free(kind, orc):
    mesh, *_ = cases.make(kind, 2)
    colour, nc = orc.colouring(mesh)
    assert colour.min() == 0 and colour.max() == nc - 1
    for c in range(nc):
        nodes = mesh.conn[colour == c].ravel()
        assert len(np.unique(nodes)) == len(nodes)


def test_uniform_rest_state_has_zero_interior_residual(gm, orc, syn):
    """Uniform p, T, Y at rest without gravity: every interior-node residual row vanishes
    (the per-element pressure terms cancel in assembly), P = I."""
    mesh = syn.channel_tri(12, 6)
    mat = syn.material_for(2, 0)
    setup = gm.Setup(2, gravity=(0.0, 0.0))
    nd = 5
    S = np.zeros((mesh.n_nodes, nd))
    S[:, 0], S[:, 3], S[:, 4] = 5e6, 1200.0, 0.8
    I = S.ravel()
    nrp, ncol, rp, col = orc.pattern(mesh, nd)
    vals, rhs, s, _ = orc.assemble(mesh, mat, setup, I, I.copy(), 1e-3, rp, col)
    interior = np.repeat(mesh.node_flag == 0, nd)
    scale = 5e6 * 12                                   # p * |grad N| * area-ish
    assert s == 0
    assert np.abs(rhs[interior]).max() < 1e-9 * scale


def test_hydrostatic_balance(gm, orc, syn):
    """p = p0 - rho g y with v = 0 and a single incompressible-ish melt: the interior
    momentum residual vanishes up to the linear-p quadrature error (exactly zero)."""
    mesh = syn.channel_tri(10, 10, Lx=1.0, Ly=1.0)
    melt = gm.custom_chemical(2400.0, 1e3, 1200.0, 1.5, 0.0, 0.0)
    mat = gm.Material([melt])
    setup = gm.Setup(2, gravity=(0.0, -9.81), dc_2006=False)
    nd = 4
    S = np.zeros((mesh.n_nodes, nd))
    S[:, 0] = 1e7 - 2400.0 * 9.81 * mesh.coords[:, 1]
    S[:, 3] = 1300.0
    I = S.ravel()
    nrp, ncol, rp, col = orc.pattern(mesh, nd)
    _, rhs, s, _ = orc.assemble(mesh, mat, setup, I, I.copy(), 1e-3, rp, col, want_matrix=False)
    interior = mesh.node_flag == 0
    mom = rhs.reshape(-1, nd)[interior][:, 1:3]
    assert s == 0
    assert np.abs(mom).max() < 1e-9 * 2400.0 * 9.81 * 0.01


def test_residual_only_equals_full(orc):
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    nd = 7
    nrp, ncol, rp, col = orc.pattern(mesh, nd)
    _, r1, _, _ = orc.assemble(mesh, mat, setup, I, P, dt, rp, col)
    _, r2, _, _ = orc.assemble(mesh, mat, setup, I, P, dt, rp, col, want_matrix=False)
    assert np.array_equal(r1, r2)


def test_coloured_threads_match_serial(orc):
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    nrp, ncol, rp, col = orc.pattern(mesh, 7)
    colour, nc = orc.colouring(mesh)
    v1, r1, _, _ = orc.assemble(mesh, mat, setup, I, P, dt, rp, col)
    v2, r2, _, _ = orc.assemble(mesh, mat, setup, I, P, dt, rp, col, nthreads=4, colour=colour, n_colours=nc)
    assert cases.rel(v2, v1) < 1e-14 and cases.rel(r2, r1) < 1e-14


def test_dirichlet_rows_and_average(gm, orc):
    """scatter.hpp:62-78: constrained rows are zero except the diagonal, which holds the
    (1 + trace)/n average of each scatter pass; their rhs entries are zero."""
    mesh, mat, setup, I, P, dt = cases.make("tri", 2, T_everywhere=True)
    nd = 5
    nrp, ncol, rp, col = orc.pattern(mesh, nd)
    vals, rhs, s, _ = orc.assemble(mesh, mat, setup, I, P, dt, rp, col)
    import scipy.sparse as sp
    A = sp.csr_matrix((vals, col, rp), shape=(len(rp) - 1,) * 2).toarray()
    T_rows = np.arange(mesh.n_nodes) * nd + 3
    assert np.all(rhs[T_rows] == 0.0)
    off = A[T_rows].copy()
    off[np.arange(len(T_rows)), T_rows] = 0.0
    assert np.all(off == 0.0)
    assert np.all(np.diag(A)[T_rows] != 0.0)
