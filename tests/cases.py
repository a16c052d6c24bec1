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
