"""Adaptive time step (adaptive_time_criteria::f_mc and set_dt, adaptive_time_step.hpp:
183-260, 380-393): the GPU per-element values against the oracle bit for bit, and the
step update against its restatement."""
import numpy as np
import pytest

import cases
from cases import gm

import oracle


@pytest.mark.parametrize("dt_el_min, dt, dt_min, dt_max", [
    (0.5, 0.1, 0.01, 1.0),     # growth bounded by 1%
    (0.05, 0.1, 0.01, 1.0),    # shrink to the element minimum
    (0.001, 0.1, 0.01, 1.0),   # clamped below
    (5.0, 2.0, 0.01, 1.0),     # clamped above
    (0.101, 0.1, 0.01, 1.0),   # exactly at the bound: 1.01 dt is not exceeded
    (1.0e30, 0.3, 0.01, 0.5),
])
def test_dt_update_matches_set_dt(dt_el_min, dt, dt_min, dt_max):
    assert gm.dt_update(dt_el_min, dt, dt_min, dt_max) == oracle.set_dt(dt_el_min, dt, dt_min, dt_max)


def _states(mesh, nc, I):
    """The seeded state, the same at rest, and one fast enough for Mach > 0.3 in gas."""
    nd = gm.nb_dofs(mesh.dim, nc)
    rest = I.copy().reshape(-1, nd)
    rest[:, 1:1 + mesh.dim] = 0.0
    fast = I.copy().reshape(-1, nd)
    fast[:, 1:1 + mesh.dim] *= 4.0e3
    return {"seeded": I, "rest": rest.ravel(), "fast": fast.ravel()}


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", [("tri", 2), ("quad", 1), ("tet", 3), ("hex", 2), ("tet", 1)])
def test_adaptive_dt_matches_oracle(kind, nc, cuda_lib):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    cfl, dt_min, dt_max = 0.5, 1e-6, 10.0
    for name, st in _states(mesh, nc, I).items():
        ref = oracle.adaptive_dt(mesh, mat, setup, st, dt, cfl)
        got = np.zeros(mesh.n_elements)
        dt_new = fa.adaptive_dt(st, dt, cfl, dt_min, dt_max, dt_el=got)
        assert np.array_equal(got, ref), (name, np.max(np.abs(got - ref) / np.abs(ref)))
        assert dt_new == oracle.set_dt(ref.min(), dt, dt_min, dt_max), name
        if name == "rest":
            assert np.all(got == 1.2 * dt)


@pytest.mark.gpu
def test_adaptive_dt_device_buffers(cuda_lib):
    torch = pytest.importorskip("torch")
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    dev = torch.device("cuda:0")
    d_el = torch.zeros(mesh.n_elements, dtype=torch.float64, device=dev)
    dt_new = fa.adaptive_dt(torch.tensor(I, device=dev), dt, 0.5, 1e-6, 10.0, dt_el=d_el)
    ref = oracle.adaptive_dt(mesh, mat, setup, I, dt, 0.5)
    assert np.array_equal(d_el.cpu().numpy(), ref)
    assert dt_new == oracle.set_dt(ref.min(), dt, 1e-6, 10.0)


@pytest.mark.gpu
@pytest.mark.parametrize("kind, nc", [("tri", 2), ("tet", 3), ("hex", 4)])
def test_secondary_dofs_match_oracle_properties(kind, nc, cuda_lib):
    """secondary_dofs::execute (secondary_dofs.hpp:56-101): the mixture at every node,
    bit for bit with the oracle's properties (fluid_properties.hpp:199-227)."""
    mesh, mat, setup, I, P, dt = cases.make(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    got = fa.secondary_dofs(I)
    nd, dim = fa.nd, mesh.dim
    S = I.reshape(-1, nd)
    keys = ["rho", "mu", "cp", "cv", "alpha", "beta", "kappa", "c"]
    for node in range(0, mesh.n_nodes, max(1, mesh.n_nodes // 97)):
        Y = np.zeros(nc)
        Y[:nc - 1] = S[node, dim + 2:]
        s = 0.0
        for i in range(nc - 1):
            s += Y[i]
        Y[nc - 1] = 1.0 - s
        ref = oracle.properties(mat, S[node, 0], S[node, dim + 1], Y)
        assert np.array_equal(got[:, node], np.array([ref[k] for k in keys])), node
