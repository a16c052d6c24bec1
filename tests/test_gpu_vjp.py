"""Vector-Jacobian products of the assembled rhs on the GPU.

FROZEN: g = A^T lambda with A the assembled FP64 tangent (checked against the CSR
matrix the same handle assembles).
EXACT: g = (db/dI)^T lambda and (db/dtheta)^T lambda, checked against central finite
differences of the FP64 residual through the C ABI (step 1e-6 relative for the
state, 1e-2..1e-4 fourth-order for the parameters), and through the
torch.autograd.Function harness.

The residual is piecewise smooth (min() in tau's caps and its time scale, |.| in the
dc length scale), so a difference step is taken from a short list (state: 1e-6 and
1e-7; parameters: 1e-2 down to 1e-6) and the check passes when one of them agrees.

States for the exact checks keep a nonzero wall velocity: on an element whose
velocity field is rank one (every node but one on a no-slip wall) compute_h takes a
branch decided by rounding noise (quad.hpp:367-375), where the residual is not
differentiable and differences straddle the branch.
"""
import numpy as np
import pytest

import cases
from cases import gm, syn, rel

import autograd_harness as ah


def _case(kind, nc, seed=0, no_slip=True):
    mesh, mat, setup, I, P, dt = cases.make(kind, nc, seed=seed)
    if not no_slip:
        I, P = syn.state_for(mesh, nc, seed, perturb=1e-4, no_slip_flag=-1)
    # parameters round-tripped through the VJP parameterisation
    mat = ah.material_from_theta(mat, ah.theta_of(mat))
    return mesh, mat, setup, I, P, dt


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", [("tet", 3), ("tri", 2), ("hex", 4), ("quad", 3)])
def test_frozen_vjp_is_transpose_of_assembled_tangent(kind, nc, cuda_lib):
    mesh, mat, setup, I, P, dt = _case(kind, nc)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lp = fa.linear_system()
    fa.execute(I, P, dt, lp, form=gm.FORM_FP64)
    A = lp.matrix_scipy()
    lam = np.random.default_rng(3).normal(size=fa.n_rows)
    g = np.zeros(fa.n_rows)
    fa.vjp(I, P, dt, lam, gm.VJP_FROZEN, g)
    assert rel(g, A.T @ lam) <= 1e-12


def _lb(fa, I, P, dt, lam):
    b = np.zeros(fa.n_rows)
    fa.residual(I, P, dt, b, form=gm.FORM_FP64)
    return float(lam @ b), float(np.abs(lam * b).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", [("tet", 3), ("tri", 2), ("hex", 4), ("tet", 1)])
def test_exact_vjp_state_matches_central_differences(kind, nc, cuda_lib):
    mesh, mat, setup, I, P, dt = _case(kind, nc, no_slip=False)
    fa = gm.FluidAssembly(mesh, mat, setup)
    rng = np.random.default_rng(11)
    lam = rng.normal(size=fa.n_rows)
    lam /= np.linalg.norm(lam)
    g = np.zeros(fa.n_rows)
    th = np.zeros(3 * nc)
    fa.vjp(I, P, dt, lam, gm.VJP_EXACT, g, th)
    scale = np.abs(I.reshape(-1, fa.nd)).max(axis=0)
    for k in range(3):
        d = (rng.normal(size=I.shape).reshape(-1, fa.nd) * scale).ravel()
        an = float(g @ d)
        # the residual has kinks (|.| in the dc length, min() in tau's caps); a direction
        # may pass one within a step of 1e-6, so a shorter step may stand in for it
        res = []
        for h in (1e-6, 1e-7):
            lp_, ap = _lb(fa, I + h * d, P, dt, lam)
            lm_, am = _lb(fa, I - h * d, P, dt, lam)
            fd = (lp_ - lm_) / (2 * h)
            noise = 10 * 2.2e-16 * max(ap, am) / h
            res.append((abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + noise, h, fd))
        assert any(r[0] for r in res), (k, an, res)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,nc", [("tet", 3), ("tri", 2)])
def test_exact_vjp_parameters_match_central_differences(kind, nc, cuda_lib):
    mesh, mat, setup, I, P, dt = _case(kind, nc, no_slip=False)
    fa = gm.FluidAssembly(mesh, mat, setup)
    lam = np.random.default_rng(12).normal(size=fa.n_rows)
    lam /= np.linalg.norm(lam)
    g = np.zeros(fa.n_rows)
    th = np.zeros(3 * nc)
    fa.vjp(I, P, dt, lam, gm.VJP_EXACT, g, th)
    theta = ah.theta_of(mat)

    def lb(t):
        f2 = gm.FluidAssembly(mesh, ah.material_from_theta(mat, t), setup)
        return _lb(f2, I, P, dt, lam)

    _, L_abs = lb(theta)
    for i in range(3 * nc):
        an = th[i] * theta[i]
        ok = []
        # weak parameters need a wide step (rounding), strong ones may pass a kink of the
        # residual (min() caps, |.|) within a wide step: the step runs from 1e-2 to 1e-6
        for h in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
            vals = []
            for m in (1, -1, 2, -2):
                t = theta.copy()
                t[i] *= 1 + m * h
                vals.append(lb(t)[0])
            fd = (8 * (vals[0] - vals[1]) - (vals[2] - vals[3])) / (12 * h)
            ok.append(abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + 10 * 2.2e-16 * L_abs / h)
        assert any(ok), (i, an)


@pytest.mark.gpu
def test_autograd_harness_backward_matches_differences(cuda_lib):
    torch = pytest.importorskip("torch")
    mesh, mat, setup, I, P, dt = _case("tet", 3, no_slip=False)
    dev = torch.device("cuda:0")
    It = torch.tensor(I, device=dev, requires_grad=True)
    theta = torch.tensor(ah.theta_of(mat), device=dev, requires_grad=True)
    Pt = torch.tensor(P, device=dev)
    w = torch.tensor(np.random.default_rng(5).normal(size=I.size), device=dev)
    b = ah.GalesRhs.apply(It, theta, mesh, mat, setup, Pt, dt)
    (b * w).sum().backward()
    nd = I.size // len(mesh.coords)
    scale = np.tile(np.abs(I.reshape(-1, nd)).max(axis=0), len(mesh.coords))
    d = torch.tensor(np.random.default_rng(6).normal(size=I.size) * scale, device=dev)
    h = 1e-6
    with torch.no_grad():
        bp = ah.GalesRhs.apply(It + h * d, theta, mesh, mat, setup, Pt, dt)
        bm = ah.GalesRhs.apply(It - h * d, theta, mesh, mat, setup, Pt, dt)
    fd = float(((bp - bm) * w).sum() / (2 * h))
    an = float((It.grad * d).sum())
    noise = 10 * 2.2e-16 * float((bp * w).abs().sum()) / h
    assert abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + noise
    assert theta.grad is not None and torch.isfinite(theta.grad).all()


@pytest.mark.gpu
def test_norm2_matches_numpy(cuda_lib):
    mesh, mat, setup, I, P, dt = _case("tet", 3)
    fa = gm.FluidAssembly(mesh, mat, setup)
    b = np.zeros(fa.n_rows)
    fa.residual(I, P, dt, b, form=gm.FORM_FP64)
    assert abs(fa.norm2(b) - np.linalg.norm(b)) <= 1e-13 * np.linalg.norm(b)
