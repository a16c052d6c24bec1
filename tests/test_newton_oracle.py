"""Newton convergence of the reference's own algorithm, on the CPU oracle alone.

The reference's tangent (fluid_2d.hpp:253-331) differentiates every term of the
residual except the stabilisation parameter tau and the dc viscosity, which enter
frozen.  With the non-diagonal tau of the shipped setup (tau_non_diag_comp_2019,
tau = DUDY^-1 diag(...), fluid_2d.hpp:932-960) the state dependence left out of the
tangent is large enough that the iteration of one time step (main.cpp:216-245)
stalls: the relative residual stops near 1e-3 on a 3D near-rest state, with the
oracle's own assembly and flexible GMRES + ILU(1) on the host and no GPU involved.
The diagonal tau variants (2007, 2014) and tau off converge to the reference's
criterion ||b|| <= 1e-8 ||b_0|| in a few iterations.  The GPU loops are compared with
these histories in test_gpu_newton.py.
"""
import pytest

import cases
from cases import gm, syn


def _loop(tau, max_it, dc=True):
    mesh, nc = syn.box_tet_delaunay(8, seed=1), 3
    mat = syn.material_for(nc, 0)
    setup = syn.setup_for(3, nc, tau=tau, dc_2006=dc)
    I0, _ = syn.state_near_rest(mesh, nc, 0)
    return cases.oracle_newton(mesh, mat, setup, I0, 1e-3, max_it, (5, 6))


def test_shipped_tau_stalls_in_the_reference_loop():
    r = _loop(gm.TAU_2019, 8)
    assert not r["converged"]
    assert min(r["history"][2:]) > 1e-4, r["history"]


@pytest.mark.parametrize("tau", [gm.TAU_2007, gm.TAU_2014])
def test_diagonal_tau_converges_in_the_reference_loop(tau):
    r = _loop(tau, 8)
    assert r["converged"] and r["iterations"] <= 5, r["history"]
    assert r["history"][-1] <= 1e-8
