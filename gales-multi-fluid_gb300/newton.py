"""Newton iterations of one time step, as the reference's driver runs them.

sim/fluid_mc/P0/main.cpp:212-244: the predictor copies the last corrected state to
the previous level (P = I, fluid_updater.hpp:18-21); each iteration assembles A and
b (fluid_assembly::execute), checks ||b|| against iteration 0
(residual_check.hpp:42-80: converged when ||b|| <= max(1e-8 ||b_0||, 1e-5)), solves
A dI = b and corrects I += dI (fluid_updater.hpp:23-26), then clamps the mass
fractions into [0, 1] (model.hpp:176-184, dof_trimmer).

time_step runs the assembly on the GPU and a host linear solve (scipy GMRES with an
incomplete LU); time_step_device keeps the whole loop on the GPU: the assembly, the
residual norm, the library's flexible GMRES with ILU(k) on the device CSR values (the
reference's Belos/Ifpack solve) and the corrector with the dof trimmer, so that only
scalars cross to the host.

The tangent and the residual may come from different forms.  Newton tolerates an
approximate tangent but not an approximate residual: with the mixed form's FP32
element integrals the residual of a nearly converged state is dominated by the
rounding of large cancelling terms (absolute pressure in the momentum flux, rho E
in the energy flux, and the dc viscosity built from them), and the iteration
stalls near 1e-6..1e-4 relative.  With the mixed tangent and an FP64 residual
(residual_form=FORM_FP64) it follows the FP64 iteration to the same count.
"""
from __future__ import annotations

import numpy as np


def gmres_ilu(A, b, rtol: float = 1e-12, restart: int = 200, maxiter: int = 20, drop_tol: float = 1e-8,
              fill_factor: float = 20.0):
    """Solve A x = b with ILU-preconditioned restarted GMRES; returns (x, info)."""
    import scipy.sparse.linalg as sla
    ilu = sla.spilu(A.tocsc(), drop_tol=drop_tol, fill_factor=fill_factor)
    M = sla.LinearOperator(A.shape, ilu.solve)
    return sla.gmres(A, b, M=M, rtol=rtol, restart=restart, maxiter=maxiter)


def time_step(fa, I_prev: np.ndarray, dt: float, form: int, max_it: int = 20, trim_mass_fractions: bool = True,
              solver=gmres_ilu, residual_form=None) -> dict:
    """One time step from the converged state I_prev: the tangent from `form`, the
    residual from `residual_form` (default: the same form).  Returns the iteration
    at which the residual check passed (the reference's it_count), the relative
    residual history and the final state."""
    import importlib
    gm = importlib.import_module("gales-multi-fluid_gb300")
    nd, dim = fa.nd, fa.dim
    P = np.array(I_prev, dtype=np.float64, copy=True)
    I = P.copy()
    lp = fa.linear_system()
    rhs = np.zeros(fa.n_rows) if residual_form is not None and residual_form != form else None
    check = gm.ResidualCheck()
    history = []
    for it in range(max_it):
        fa.execute(I, P, dt, lp, form=form)
        if rhs is not None:
            fa.residual(I, P, dt, rhs, form=residual_form)
            lp.rhs[:] = rhs
        converged, res = check.execute(lp.rhs, it)
        history.append(1.0 if it == 0 else res)
        if converged:
            return {"converged": True, "iterations": it, "history": history, "state": I}
        dx, info = solver(lp.matrix_scipy(), lp.rhs)
        I = I + dx
        if trim_mass_fractions:
            S = I.reshape(-1, nd)
            np.clip(S[:, dim + 2:], 0.0, 1.0, out=S[:, dim + 2:])
    return {"converged": False, "iterations": max_it, "history": history, "state": I}


def time_step_device(fa, solver, I_prev, dt: float, form: int, max_it: int = 3, trim=None, residual_form=None,
                     lp=None) -> dict:
    """One time step of main.cpp:216-245 on the GPU from the converged device state
    I_prev (a float64 cuda tensor): predictor P = I; per iteration the assembly, the
    residual check on ||b|| (FluidAssembly.norm2), the solve (LinearSolver) and the
    corrector I += dx followed by dof_trimmer on the dof range `trim` (default: dof
    dim + 2, the first mass fraction, to [0, 1], as main.cpp:235 trims dof 4 of the 2D
    cases).  max_it is setup.txt's n_max_it.  Returns the iteration at which the check
    passed, the relative residuals, the solver's iteration counts and the state."""
    import importlib
    import torch
    gm = importlib.import_module("gales-multi-fluid_gb300")
    dev = I_prev.device
    P = I_prev.clone()
    I = P.clone()
    if lp is None:
        lp = fa.device_system(dev)
    x = torch.zeros(fa.n_rows, dtype=torch.float64, device=dev)
    rhs = torch.zeros_like(x) if residual_form is not None and residual_form != form else None
    if trim is None:
        trim = (fa.dim + 2, fa.dim + 3) if fa.nb_comp > 1 else (-1, -1)
    check = gm.ResidualCheck()
    history, lin_its = [], []
    for it in range(max_it):
        fa.execute(I, P, dt, lp, form=form)
        if rhs is not None:
            fa.residual(I, P, dt, rhs, form=residual_form)
            lp.rhs.copy_(rhs)
        converged, res = check.execute(None, it, norm=fa.norm2(lp.rhs))
        history.append(1.0 if it == 0 else res)
        if converged:
            return {"converged": True, "iterations": it, "history": history, "linear_iterations": lin_its,
                    "state": I}
        solver.solve(lp.vals, lp.rhs, x)
        lin_its.append(solver.num_it)
        solver.correct(I, x, trim)
    return {"converged": False, "iterations": max_it, "history": history, "linear_iterations": lin_its,
            "state": I}
