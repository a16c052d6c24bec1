"""Linear solve of the assembled system (belos_linear_solver::execute,
belos_linear_solver_factory.hpp:103-218, with Flexible GMRES and Ifpack ILU as
sim/fluid_mc/P0/setup.txt:10-16 selects) and the Newton loop around it
(main.cpp:216-245).

CPU: the library's node-level ILU(k) pattern equals the oracle's scalar ILU(k) pattern
expanded by blocks, the level sets are dependency levels, and the oracle's solver
agrees with a direct solve.  GPU: the factor against the oracle's scalar factor, the
preconditioner application, the FGMRES iteration counts and solutions, and a Newton
time step on the device against the oracle's on the host.
"""
import importlib

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import cases
from cases import gm, syn

import oracle

newton = importlib.import_module("gales-multi-fluid_gb300.newton")

KINDS = [("tri", 2), ("quad", 1), ("tet", 3), ("hex", 2)]


def _system(kind, nc, seed=0):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc, seed=seed)
    nd = gm.nb_dofs(mesh.dim, nc)
    nrp, ncol, rp, col = oracle.pattern(mesh, nd)
    vals, rhs, s, _ = oracle.assemble(mesh, mat, setup, I, P, dt, rp, col)
    assert s == 0
    return mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs


def _expand(nrp, ncol, nd):
    """Scalar CSR pattern of a node-block pattern (dense nd x nd blocks)."""
    n = len(nrp) - 1
    rows, cols = [], []
    for i in range(n):
        cs = ncol[nrp[i]:nrp[i + 1]]
        sc = (cs[:, None] * nd + np.arange(nd)[None, :]).ravel()
        for k in range(nd):
            rows.append(np.full(len(sc), i * nd + k))
            cols.append(sc)
    r, c = np.concatenate(rows), np.concatenate(cols)
    rp = np.zeros(n * nd + 1, dtype=np.int64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp), c.astype(np.int32)


def _blocks_to_csr(f_rp, f_col, blocks, nd):
    n = len(f_rp) - 1
    data, rows, cols = [], [], []
    for i in range(n):
        for p in range(f_rp[i], f_rp[i + 1]):
            J = f_col[p]
            for r in range(nd):
                rows.append(np.full(nd, i * nd + r))
                cols.append(J * nd + np.arange(nd))
                data.append(blocks[p, r])
    return sp.csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))), shape=(n * nd,) * 2)


@pytest.mark.parametrize("kind, nc", KINDS)
@pytest.mark.parametrize("fill", [0, 1, 2])
def test_node_pattern_is_scalar_pattern(kind, nc, fill):
    """Scalar ILU(k) of the block-dense assembled pattern (the oracle, Ifpack_IlukGraph's
    rule) has exactly the node-level ILU(k) pattern expanded by blocks."""
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    nd = gm.nb_dofs(mesh.dim, nc)
    nrp, ncol, rp, col = oracle.pattern(mesh, nd)
    f_rp, f_col, lf, lb, nl = gm.iluk_pattern(nrp, ncol, fill)
    s_rp, s_col, _, _ = oracle.iluk(rp, col, np.ones(len(col)), fill)
    e_rp, e_col = _expand(f_rp, f_col, nd)
    assert np.array_equal(e_rp, s_rp)
    assert np.array_equal(e_col, s_col)
    # the pattern contains the graph and is sorted with a diagonal in every row
    for i in range(len(nrp) - 1):
        row = f_col[f_rp[i]:f_rp[i + 1]]
        assert np.all(np.diff(row) > 0) and i in row
        assert set(ncol[nrp[i]:nrp[i + 1]]) <= set(row)
    # levels: a row's forward level is one more than its lower columns' maximum
    for i in range(len(nrp) - 1):
        row = f_col[f_rp[i]:f_rp[i + 1]]
        lo, hi = row[row < i], row[row > i]
        assert lf[i] == (lf[lo].max() + 1 if len(lo) else 0)
        assert lb[i] == (lb[hi].max() + 1 if len(hi) else 0)
    assert nl == (lf.max() + 1, lb.max() + 1)


def test_iluk_pattern_of_a_path_graph():
    """Tridiagonal node graph: no fill at any level, n forward and backward levels."""
    n = 6
    rp = [0]
    col = []
    for i in range(n):
        c = [j for j in (i - 1, i, i + 1) if 0 <= j < n]
        col += c
        rp.append(len(col))
    f_rp, f_col, lf, lb, nl = gm.iluk_pattern(np.array(rp), np.array(col), 3)
    assert np.array_equal(f_rp, rp) and np.array_equal(f_col, col)
    assert list(lf) == list(range(n)) and list(lb) == list(range(n - 1, -1, -1)) and nl == (n, n)


def test_iluk_fill_of_an_arrow_graph():
    """Row 0 couples to every node: ILU(0) keeps the graph, ILU(1) fills the whole
    trailing block (level 1 through node 0)."""
    n = 5
    rows = [[0, 1, 2, 3, 4]] + [[0, i] for i in range(1, n)]
    rp = np.cumsum([0] + [len(r) for r in rows])
    col = np.concatenate(rows)
    f_rp, f_col, *_ = gm.iluk_pattern(rp, col, 0)
    assert np.array_equal(f_col, col)
    f_rp, f_col, lf, lb, nl = gm.iluk_pattern(rp, col, 1)
    assert np.array_equal(f_rp, np.arange(0, n * n + 1, n)) and nl == (n, n)


@pytest.mark.parametrize("kind, nc", KINDS)
def test_oracle_solver_against_direct_solve(kind, nc):
    """The oracle's ILU(1) satisfies (LU)_ij = a_ij on its pattern and its FGMRES reaches
    the direct solution within the 1e-9 relative residual."""
    *_, nd, nrp, ncol, rp, col, vals, rhs = _system(kind, nc)
    n = len(rp) - 1
    A = sp.csr_matrix((vals, col, rp), shape=(n, n))
    f_rp, f_col, f_val, bad = oracle.iluk(rp, col, vals, 1)
    assert bad == -1
    F = sp.csr_matrix((f_val, f_col, f_rp), shape=(n, n))
    LU = ((sp.tril(F, -1) + sp.eye(n)) @ sp.triu(F)).tocsr()
    mask = F.copy()
    mask.data[:] = 1.0
    assert abs((LU - A).multiply(mask)).max() <= 1e-13 * abs(A).max()
    x, info = oracle.fgmres(rp, col, vals, rhs)
    assert info["converged"] and info["rel_res"] <= 1e-9 and info["cycles"] == 1
    xd = sla.spsolve(A.tocsc(), rhs)
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)
    # at convergence ||b - A x|| ~ 1e-10 ||b||: recomputing it in another summation order
    # is accurate to ~eps ||A|| ||x|| / ||b - A x|| ~ 1e-6 relative
    assert np.linalg.norm(rhs - A @ x) == pytest.approx(info["abs_res"], rel=1e-4)


# ---------------------------------------------------------------------------
# GPU


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", KINDS)
@pytest.mark.parametrize("fill", [0, 1, 2])
def test_factor_matches_oracle(kind, nc, fill, cuda_lib):
    mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs = _system(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver(gm.SolverParams(fill=fill))
    sol.factorize(vals)
    f_rp, f_col, blocks = sol.factor()
    G = _blocks_to_csr(f_rp, f_col, blocks, nd)
    s_rp, s_col, s_val, bad = oracle.iluk(rp, col, vals, fill)
    assert bad == -1
    assert np.array_equal(G.indptr, s_rp) and np.array_equal(G.indices, s_col)
    scale = np.abs(s_val).max()
    assert np.max(np.abs(G.data - s_val)) <= 1e-13 * scale


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", KINDS)
def test_factor_is_bitwise_scalar_elimination(kind, nc, cuda_lib):
    """The block factorisation performs the scalar ikj elimination's operations in its
    order: the factor equals the oracle's bit for bit."""
    mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs = _system(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver()
    sol.factorize(vals)
    G = _blocks_to_csr(*sol.factor(), nd)
    _, _, s_val, _ = oracle.iluk(rp, col, vals, 1)
    assert np.array_equal(G.data, s_val)


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", KINDS)
def test_preconditioner_apply_matches_oracle(kind, nc, cuda_lib):
    import torch
    mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs = _system(kind, nc)
    n = len(rp) - 1
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver()
    sol.factorize(vals)
    v = np.random.default_rng(3).standard_normal(n)
    dv = torch.tensor(v, device="cuda:0")
    dz = torch.zeros_like(dv)
    sol.apply(dv, dz)
    torch.cuda.synchronize()
    s_rp, s_col, s_val, _ = oracle.iluk(rp, col, vals, 1)
    F = sp.csr_matrix((s_val, s_col, s_rp), shape=(n, n))
    y = sla.spsolve_triangular((sp.tril(F, -1) + sp.eye(n)).tocsr(), v, lower=True)
    z = sla.spsolve_triangular(sp.triu(F).tocsr(), y, lower=False)
    assert np.linalg.norm(dz.cpu().numpy() - z) <= 1e-12 * np.linalg.norm(z)


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", KINDS)
def test_fgmres_matches_oracle(kind, nc, cuda_lib):
    mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs = _system(kind, nc)
    n = len(rp) - 1
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver()
    x = np.zeros(n)
    sol.solve(vals, rhs, x)
    xo, info = oracle.fgmres(rp, col, vals, rhs)
    assert sol.converged and sol.RRE <= 1e-9
    assert abs(sol.num_it - info["iterations"]) <= 1, (sol.num_it, info)
    assert sol.result.cycles == info["cycles"]
    A = sp.csr_matrix((vals, col, rp), shape=(n, n))
    assert np.linalg.norm(rhs - A @ x) == pytest.approx(sol.ARE, rel=1e-4)
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", KINDS)
def test_fp32_preconditioner(kind, nc, cuda_lib):
    """The ILU in FP32 (factor and substitutions) under the FP64 Krylov iteration: the
    factor's significant entries agree with the oracle's FP64 factor to the FP32
    rounding the elimination amplifies (up to 6e-3 relative measured on the quad case,
    1e-3 on the others) and the solve reaches the same tolerance in the FP64 factor's
    iteration count (within two)."""
    mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs = _system(kind, nc)
    n = len(rp) - 1
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver(gm.SolverParams(precond=gm.PRECOND_ILU_FP32))
    sol.factorize(vals)
    G = _blocks_to_csr(*sol.factor(), nd)
    _, _, s_val, _ = oracle.iluk(rp, col, vals, 1)
    big = np.abs(s_val) > 1e-3 * np.abs(s_val).max()
    assert np.max(np.abs(G.data - s_val)[big] / np.abs(s_val)[big]) <= 2e-2
    x = np.zeros(n)
    sol.solve(vals, rhs, x)
    xo, info = oracle.fgmres(rp, col, vals, rhs)
    assert sol.converged and sol.RRE <= 1e-9
    assert abs(sol.num_it - info["iterations"]) <= 2, (sol.num_it, info)
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)


@pytest.mark.gpu
def test_fgmres_device_buffers_and_repeatability(cuda_lib):
    """Device CSR values from the assembly, as the Newton loop passes them; two solves
    give identical bits; host and device buffers give the same solution."""
    import torch
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.device_system("cuda:0")
    dI, dP = torch.tensor(I, device="cuda:0"), torch.tensor(P, device="cuda:0")
    fa.execute(dI, dP, dt, lp, form=gm.FORM_FP64)
    sol = fa.linear_solver()
    x1 = torch.zeros(fa.n_rows, dtype=torch.float64, device="cuda:0")
    x2 = torch.zeros_like(x1)
    sol.solve(lp.vals, lp.rhs, x1)
    it1 = sol.num_it
    sol.solve(lp.vals, lp.rhs, x2)
    assert sol.num_it == it1 and torch.equal(x1, x2)
    xh = np.zeros(fa.n_rows)
    sol.solve(lp.vals.cpu().numpy(), lp.rhs.cpu().numpy(), xh)
    assert np.array_equal(xh, x1.cpu().numpy())
    assert sol.launch_count() > 0


@pytest.mark.gpu
def test_unpreconditioned_and_restarted_gmres_match_oracle(cuda_lib):
    """precond NONE and a short restart length (several cycles) follow the oracle's
    iteration and cycle counts."""
    mesh, mat, setup, I, P, dt, nd, nrp, ncol, rp, col, vals, rhs = _system("quad", 1)
    n = len(rp) - 1
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver(gm.SolverParams(maxsubspace=5, maxrestarts=3, fill=0))
    x = np.zeros(n)
    sol.solve(vals, rhs, x)
    xo, info = oracle.fgmres(rp, col, vals, rhs, maxsubspace=5, maxrestarts=3, fill=0)
    assert sol.result.cycles == info["cycles"] and abs(sol.num_it - info["iterations"]) <= 1
    assert sol.converged == info["converged"]
    sol = fa.linear_solver(gm.SolverParams(precond=gm.PRECOND_NONE, maxiters=40, maxsubspace=20))
    sol.solve(vals, rhs, x)
    xo, info = oracle.fgmres(rp, col, vals, rhs, precond=False, maxiters=40, maxsubspace=20)
    assert sol.num_it == info["iterations"] == 40 and not sol.converged
    assert sol.RRE == pytest.approx(info["rel_res"], rel=1e-3)


@pytest.mark.gpu
def test_correct_trims_one_dof(cuda_lib):
    import torch
    mesh, mat, setup, I, P, dt = cases.make("tri", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver(gm.SolverParams(precond=gm.PRECOND_NONE, maxsubspace=2))
    nd = fa.nd
    dI = torch.tensor(I, device="cuda:0")
    dx = torch.zeros_like(dI)
    dx.view(-1, nd)[:, 4] = 2.0
    dx.view(-1, nd)[:, 5] = -3.0
    sol.correct(dI, dx, (4, 5), 0.0, 1.0)
    torch.cuda.synchronize()
    ref = I.copy().reshape(-1, nd) + dx.cpu().numpy().reshape(-1, nd)
    ref[:, 4] = np.maximum(0.0, np.minimum(ref[:, 4], 1.0))
    assert np.array_equal(dI.cpu().numpy().reshape(-1, nd), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", [("quad", 1), ("hex", 2)])
def test_newton_on_device_matches_oracle(kind, nc, cuda_lib):
    """main.cpp:216-245 with the shipped n_max_it = 3: the assembly, the residual check,
    the solve and the corrector on the GPU follow the oracle's loop (assembly, FGMRES
    with ILU(1), corrector and dof trimmer on the host): the same convergence decisions,
    Krylov iteration counts within one, residual histories and states to the solve
    tolerance."""
    import torch
    mesh, mat, setup, I0, P0, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver()
    trim = (mesh.dim + 2, mesh.dim + 3) if nc > 1 else (0, 0)
    dev = newton.time_step_device(fa, sol, torch.tensor(I0, device="cuda:0"), dt, gm.FORM_FP64, max_it=3,
                                  trim=trim)
    ref = cases.oracle_newton(mesh, mat, setup, I0, dt, 3, trim)
    assert dev["converged"] == ref["converged"] and dev["iterations"] == ref["iterations"]
    assert ref["history"][-1] < 0.5  # the iteration makes progress on this state
    assert np.allclose(dev["history"], ref["history"], rtol=1e-5, atol=0)
    assert all(abs(a - b) <= 1 for a, b in zip(dev["linear_iterations"], ref["linear_iterations"])), \
        (dev["linear_iterations"], ref["linear_iterations"])
    S, R = dev["state"].cpu().numpy(), ref["state"]
    assert np.linalg.norm(S - R) <= 1e-6 * np.linalg.norm(R)


@pytest.mark.gpu
def test_newton_device_loop_equals_host_loop(cuda_lib):
    """The device-resident loop (norm on the device, corrector kernel) follows the host
    loop driving the same GPU solver through host arrays.  The atomic scatter adds the
    element blocks in a run-dependent order, so the two assemblies agree to rounding,
    which the solves amplify by the system's conditioning."""
    import torch
    mesh, mat, setup, I0, P0, dt = cases.make("hex", 2)
    fa = gm.FluidAssembly(mesh, mat, setup)
    sol = fa.linear_solver()

    def gpu_solve(A, b):
        x = np.zeros(len(b))
        sol.solve(np.ascontiguousarray(A.data), np.ascontiguousarray(b), x)
        return x, 0

    host = newton.time_step(fa, I0, dt, gm.FORM_FP64, max_it=3, solver=gpu_solve)
    dev = newton.time_step_device(fa, sol, torch.tensor(I0, device="cuda:0"), dt, gm.FORM_FP64, max_it=3,
                                  trim=(mesh.dim + 2, fa.nd))
    # the residual norms differ only in summation order (numpy on the host, blocked sums on
    # the device)
    assert host["iterations"] == dev["iterations"]
    assert np.allclose(host["history"], dev["history"], rtol=1e-8, atol=0)
    S, R = dev["state"].cpu().numpy(), host["state"]
    assert np.linalg.norm(S - R) <= 1e-8 * np.linalg.norm(R)


def _iluk_python(n, rows, fill):
    """Level-of-fill ILU(k) pattern, written directly from the rule (dicts per row)."""
    pat = []
    for i in range(n):
        lev = {j: 0 for j in rows[i]}
        lev.setdefault(i, 0)
        k = min(lev)
        while k < i:
            lik = lev[k]
            for j, lkj in pat[k].items():
                if j > k and lik + lkj + 1 <= fill:
                    lev[j] = min(lev.get(j, 99), lik + lkj + 1)
            k = min((c for c in lev if c > k), default=i)
        pat.append(lev)
    return pat


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("fill", [0, 1, 3])
def test_iluk_pattern_random_graphs(seed, fill):
    """The library's linked-list symbolic factorisation on irregular graphs (some rows
    without their diagonal, unsymmetric couplings) against the rule written with dicts."""
    rng = np.random.default_rng(seed)
    n = 60
    rows = []
    for i in range(n):
        c = set(rng.choice(n, size=rng.integers(1, 6), replace=False).tolist())
        if rng.random() < 0.7:
            c.add(i)
        rows.append(sorted(c))
    rp = np.cumsum([0] + [len(r) for r in rows])
    col = np.concatenate([np.array(r, dtype=np.int32) for r in rows])
    f_rp, f_col, lf, lb, nl = gm.iluk_pattern(rp, col, fill)
    ref = _iluk_python(n, rows, fill)
    for i in range(n):
        assert list(f_col[f_rp[i]:f_rp[i + 1]]) == sorted(ref[i]), i


def test_oracle_full_fill_is_exact_lu():
    """With a level of fill as large as the matrix, ILU(k) is the LU factorisation
    without pivoting: L U = A everywhere and FGMRES converges in one step to the
    direct solution (a pin of the restated elimination and of the Krylov loop)."""
    *_, nd, nrp, ncol, rp, col, vals, rhs = _system("quad", 1)
    n = len(rp) - 1
    A = sp.csr_matrix((vals, col, rp), shape=(n, n))
    f_rp, f_col, f_val, bad = oracle.iluk(rp, col, vals, n)
    assert bad == -1
    F = sp.csr_matrix((f_val, f_col, f_rp), shape=(n, n))
    LU = ((sp.tril(F, -1) + sp.eye(n)) @ sp.triu(F)).toarray()
    assert np.abs(LU - A.toarray()).max() <= 1e-11 * abs(A).max()
    x, info = oracle.fgmres(rp, col, vals, rhs, fill=n)
    assert info["iterations"] == 1 and info["converged"]
    xd = sla.spsolve(A.tocsc(), rhs)
    assert np.linalg.norm(x - xd) <= 1e-9 * np.linalg.norm(xd)


def test_oracle_ilu_values_equal_plain_python_elimination():
    """The oracle's numeric ILU(1) equals a plain-Python row-oriented (ikj) elimination
    restricted to the same pattern, bit for bit (Python floats are IEEE binary64 without
    contraction, as the oracle is compiled)."""
    mesh = syn.channel_tri(4, 2)
    nd = gm.nb_dofs(2, 2)
    nrp, ncol, rp, col = oracle.pattern(mesh, nd)
    vals, rhs, s, _ = oracle.assemble(mesh, syn.material_for(2, 0), syn.setup_for(2, 2), *syn.state_for(mesh, 2, 0),
                                      1e-3, rp, col)
    f_rp, f_col, f_val, bad = oracle.iluk(rp, col, vals, 1)
    n = len(rp) - 1
    rows = []
    for i in range(n):
        pat = [int(c) for c in f_col[f_rp[i]:f_rp[i + 1]]]
        w = {c: 0.0 for c in pat}
        for p in range(rp[i], rp[i + 1]):
            w[int(col[p])] += float(vals[p])
        for k in pat:
            if k >= i:
                break
            lik = w[k] / rows[k][k]
            w[k] = lik
            for j, u in rows[k].items():
                if j > k and j in w:
                    w[j] -= lik * u
        rows.append(w)
    ref = np.array([rows[i][int(c)] for i in range(n) for c in f_col[f_rp[i]:f_rp[i + 1]]])
    assert np.array_equal(ref, f_val)
