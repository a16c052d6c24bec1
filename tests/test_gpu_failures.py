"""Failure detection through the status word, with no GPU fault involved.

The library never traps: bad input is reported as a status bit plus the first
offending element (the reference calls Error()/MPI_Abort instead,
algorithm.hpp:37-44), and the handle stays usable afterwards.
"""
import numpy as np
import pytest

import cases
from cases import rel


@pytest.mark.gpu
def test_inverted_element_rejected_at_create(cuda_lib, gm):
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    conn = mesh.conn.copy()
    conn[7, [1, 2]] = conn[7, [2, 1]]  # negative Jacobian (quad.hpp:215-218)
    bad = gm.Mesh(mesh.coords, conn, mesh.node_flag, mesh.el_on_boundary, mesh.bd_sides)
    with pytest.raises(gm.GalesError) as ei:
        gm.FluidAssembly(bad, mat, setup)
    assert ei.value.code & gm.abi.ERR_NEG_JACOBIAN


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_nonfinite_state_reported_and_handle_survives(form, cuda_lib, gm, orc):
    f = gm.FORM_FP64 if form == "fp64" else gm.FORM_MIXED
    mesh, mat, setup, I, P, dt = cases.make("tet", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system()
    nd = fa.nd
    node = int(mesh.conn[11, 2])
    Ib = I.copy()
    Ib[node * nd + 0] = np.nan  # pressure
    with pytest.raises(gm.GalesError) as ei:
        fa.execute(Ib, P, dt, lp, form=f)
    assert ei.value.code & gm.abi.ERR_NONFINITE
    touching = np.nonzero((mesh.conn == node).any(axis=1))[0]
    assert ei.value.first_bad == touching.min()
    # the same handle assembles a finite state afterwards
    fa.execute(I, P, dt, lp, form=f)
    vals, rhs, s, _ = orc.assemble(mesh, mat, setup, I, P, dt, lp.row_ptr, lp.col)
    assert s == 0
    tol = 1e-12 if form == "fp64" else 1e-6
    assert rel(lp.vals, vals) <= tol and rel(lp.rhs, rhs) <= tol
