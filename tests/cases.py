"""Small seeded parity cases shared by the CPU and GPU tests."""
import importlib

import numpy as np

gm = importlib.import_module("gales-multi-fluid_gb300")
syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")


def make(kind: str, nc: int, seed: int = 0, setup_kw=None, T_everywhere=False, perturb=1e-4):
    setup_kw = dict(setup_kw or {})
    if kind == "tri":
        mesh = syn.channel_tri(16, 8)
    elif kind == "tri_c0":
        mesh = syn.channel_tri()
    elif kind == "quad":
        mesh = syn.channel_quad(12, 6, jitter=0.2, seed=seed)
    elif kind == "tet":
        mesh = syn.box_tet_delaunay(6, seed=seed + 1)
    elif kind == "hex":
        mesh = syn.box_hex(4, 4, 3, jitter=0.1, seed=seed + 2)
    else:
        raise KeyError(kind)
    mat = syn.material_for(nc, seed)
    setup = syn.setup_for(mesh.dim, nc, dirichlet_T_everywhere=T_everywhere, **setup_kw)
    I, P = syn.state_for(mesh, nc, seed, perturb=perturb)
    return mesh, mat, setup, I, P, 1e-3


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def oracle_newton(mesh, mat, setup, I0, dt, max_it, trim, fill=1):
    """The reference's time-step loop (main.cpp:216-245) with the oracle's assembly and
    its flexible GMRES + ILU(fill) on the host: predictor P = I, residual check
    ||b|| <= max(1e-8 ||b_0||, 1e-5) (residual_check.hpp:42-80), corrector I += dx and
    the dof trimmer on the dof range `trim`."""
    import oracle
    nd = gm.nb_dofs(mesh.dim, mat.nb_comp)
    nrp, ncol, rp, col = oracle.pattern(mesh, nd)
    P = np.array(I0, dtype=np.float64, copy=True)
    I = P.copy()
    res0, its, hist = 0.0, [], []
    for it in range(max_it):
        vals, rhs, s, _ = oracle.assemble(mesh, mat, setup, I, P, dt, rp, col)
        nb = float(np.linalg.norm(rhs))
        if it == 0:
            res0 = nb
            hist.append(1.0)
        else:
            hist.append(nb / res0)
            if nb <= max(1e-8 * res0, 1e-5):
                return dict(converged=True, iterations=it, history=hist, linear_iterations=its, state=I)
        x, info = oracle.fgmres(rp, col, vals, rhs, fill=fill)
        its.append(info["iterations"])
        I = I + x
        S = I.reshape(-1, nd)
        S[:, trim[0]:trim[1]] = np.maximum(0.0, np.minimum(S[:, trim[0]:trim[1]], 1.0))
    return dict(converged=False, iterations=max_it, history=hist, linear_iterations=its, state=I)
