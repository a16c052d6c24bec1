"""Point-level exact VJP (gales_vjp.cuh) against central finite differences, on the CPU.

The GPU adjoint kernel calls point_forward/point_reverse; here the same
__host__ __device__ code is compiled for the host and its reverse mode is checked
against differences of its forward: state, state gradient and the material
parameters (density parameter, mu, cp per component), for each tau/dc branch.
"""
import ctypes as C
import importlib
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
gm = importlib.import_module("gales-multi-fluid_gb300")
syn = importlib.import_module("gales-multi-fluid_gb300.synthetic")
R_U = 8.314462


class DevChem(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32)] + [
        (n, C.c_double) for n in ("rho", "mu", "cp", "cv", "kappa", "alpha", "beta", "R", "gamma", "D", "inv_rho",
                                  "beta_over_rho", "alpha_over_rho", "cv_shift", "inv_R", "R_over_gamma", "inv_D",
                                  "c2_coef")]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("vjp")
    so = d / "vjp_host.so"
    subprocess.run(["nvcc", "-std=c++17", "-O1", "-x", "cu", "-shared", "-Xcompiler", "-fPIC", "-o", str(so),
                    str(ROOT / "tests" / "host" / "vjp_point_host.cu")], check=True)
    return C.CDLL(str(so))


def _chems(nc, seed=0):
    mat = syn.material_for(nc, seed)
    out = (DevChem * nc)()
    for i in range(nc):
        s = mat.desc.comp[i]
        o = out[i]
        o.kind = s.kind
        for n in ("rho", "mu", "cp", "cv", "kappa", "alpha", "beta", "R", "gamma"):
            setattr(o, n, getattr(s, n))
        o.D = s.chemical_diffusivity
    return out


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Point:
    def __init__(self, lib, dim, nen, nc, seed, tau=2019, dc=1, sharp=2.0, steady=0, v_scale=0.1):
        self.lib, self.dim, self.nen, self.nc = lib, dim, nen, nc
        self.nd = dim + 1 + nc
        nd = self.nd
        rng = np.random.default_rng(seed)
        self.ch = _chems(nc, seed)
        self.scal = np.array([1e-3, sharp, 1.0, 0.0, 0.0 if dim == 3 else -9.81, -9.81 if dim == 3 else 0.0,
                              tau, dc, steady], dtype=np.float64)
        self.uri = np.abs(rng.normal(1.0, 0.2, nd)) * np.array(
            [1e-3] + [1e-2] * dim + [1e-9] + [1e-3] * (nc - 1))
        A = rng.normal(0, 1, (dim, dim))
        self.G = ((A @ A.T + dim * np.eye(dim)) * 2500.0).ravel()
        ds = rng.normal(0, 50.0, (dim, nen))
        ds -= ds.mean(axis=1, keepdims=True)
        self.ds = ds.ravel()
        Y = rng.dirichlet(np.ones(nc))
        I = np.concatenate([[5e7 * (1 + 0.01 * rng.normal())], v_scale * rng.normal(0, 1, dim),
                            [1300 + 50 * rng.normal()], Y[:-1]])
        self.I = I
        self.P = I * (1 + 1e-4 * rng.normal(0, 1, nd))
        sc = np.concatenate([[1e8], [1.0] * dim, [100.0], [1.0] * (nc - 1)])
        self.dI = (rng.normal(0, 1, (dim, nd)) * sc).ravel()
        self.phi0b = rng.normal(0, 1, nd)
        self.phib = rng.normal(0, 1, dim * nd)
        tag = f"{dim}_{nen}_{nc}"
        self.f = getattr(lib, "pt_forward_" + tag)
        self.r = getattr(lib, "pt_reverse_" + tag)

    def loss(self, I=None, dI=None, ch=None):
        I = self.I if I is None else I
        dI = self.dI if dI is None else dI
        ch = self.ch if ch is None else ch
        phi0 = np.zeros(self.nd)
        phi = np.zeros(self.dim * self.nd)
        self.f(ch, _ptr(self.scal), _ptr(self.uri), _ptr(self.G), _ptr(self.ds), _ptr(I), _ptr(dI), _ptr(self.P),
               _ptr(phi0), _ptr(phi))
        self.last_abs = float(np.abs(self.phi0b * phi0).sum() + np.abs(self.phib * phi).sum())
        return float(self.phi0b @ phi0 + self.phib @ phi)

    def grads(self):
        Ib = np.zeros(self.nd)
        dIb = np.zeros(self.dim * self.nd)
        th = np.zeros(3 * self.nc)
        self.r(self.ch, _ptr(self.scal), _ptr(self.uri), _ptr(self.G), _ptr(self.ds), _ptr(self.I), _ptr(self.dI),
               _ptr(self.P), _ptr(self.phi0b), _ptr(self.phib), _ptr(Ib), _ptr(dIb), _ptr(th))
        return Ib, dIb, th

    def perturbed_chems(self, c, k, h):
        out = (DevChem * self.nc)()
        C.memmove(out, self.ch, C.sizeof(out))
        q = out[c]
        if k == 0:
            if q.kind == gm.abi.CH_CUSTOM:
                q.rho *= 1 + h
            else:
                q.R = R_U / ((R_U / q.R) * (1 + h))
        elif k == 1:
            q.mu *= 1 + h
        else:
            q.cp *= 1 + h
        return out

    def param_value(self, c, k):
        q = self.ch[c]
        if k == 0:
            return q.rho if q.kind == gm.abi.CH_CUSTOM else R_U / q.R
        return q.mu if k == 1 else q.cp


CASES = [dict(dim=3, nen=4, nc=3), dict(dim=3, nen=4, nc=1), dict(dim=2, nen=3, nc=2), dict(dim=3, nen=8, nc=4)]
VARIANTS = [dict(), dict(sharp=1.0), dict(sharp=1.5), dict(dc=0), dict(tau=0), dict(steady=1),
            dict(v_scale=300.0)]


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['dim']}d{c['nen']}n{c['nc']}c")
@pytest.mark.parametrize("var", VARIANTS, ids=lambda v: ",".join(f"{k}={x}" for k, x in v.items()) or "default")
def test_point_vjp_matches_central_differences(lib, case, var):
    for seed in range(3):
        pt = Point(lib, seed=seed, **case, **var)
        Ib, dIb, th = pt.grads()
        rng = np.random.default_rng(100 + seed)
        # state and state gradient along random directions scaled to each entry
        for _ in range(3):
            dI_dir = rng.normal(0, 1, pt.dI.size) * np.abs(pt.dI)
            I_dir = rng.normal(0, 1, pt.nd) * np.maximum(np.abs(pt.I), 1e-3)
            h = 1e-6
            fd = (pt.loss(pt.I + h * I_dir, pt.dI + h * dI_dir) - pt.loss(pt.I - h * I_dir, pt.dI - h * dI_dir)) / (2 * h)
            an = float(Ib @ I_dir + dIb @ dI_dir)
            assert _rel(fd, an) < 1e-5, (seed, fd, an)
        # each material parameter, fourth-order central differences.  A weak parameter (a
        # gas viscosity) moves the loss by little more than the rounding of its largest
        # terms, so the bar is 1e-5 relative plus the difference quotient's own rounding
        # bound, ~1.5 eps sum|phi_bar phi| / h.
        pt.loss()
        L_abs = pt.last_abs
        for c in range(pt.nc):
            for k in range(3):
                an = th[3 * c + k] * pt.param_value(c, k)
                ok = []
                for h in (1e-2, 1e-3, 1e-4):
                    Lp = [pt.loss(ch=pt.perturbed_chems(c, k, m * h)) for m in (1, -1, 2, -2)]
                    fd = (8 * (Lp[0] - Lp[1]) - (Lp[2] - Lp[3])) / (12 * h)
                    noise = 10 * 2.2e-16 * L_abs / h
                    ok.append((abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + noise, fd))
                assert any(o for o, _ in ok), (seed, c, k, an, ok, L_abs)


def _side_bc(kind, dim, nc):
    bc = gm.abi.SideBC()
    if kind == "tau":
        bc.tau_mask = 1 << (0 * 3 + 1)
        bc.tau[1] = 3.0
    elif kind == "q":
        bc.q_mask = 1 << (dim - 1)
        bc.q[dim - 1] = 7.0
    elif kind == "J" and nc > 1:
        bc.J_mask = 1 << ((dim - 1) * 8 + 0)
        bc.J[dim - 1][0] = 1e-3
    elif kind == "mf":
        bc.mass_flux_mask = 1 << (dim - 1)
        bc.mass_flux[dim - 1] = 2.5
    return bc


@pytest.mark.parametrize("dim,nc", [(3, 3), (2, 2), (3, 4), (3, 1)])
@pytest.mark.parametrize("kind", ["none", "tau", "q", "J", "mf"])
def test_boundary_point_vjp_matches_central_differences(lib, dim, nc, kind):
    for seed in range(3):
        pt = Point(lib, dim, {(3, 3): 4, (2, 2): 3, (3, 4): 8, (3, 1): 4}[(dim, nc)], nc, seed)
        bc = _side_bc(kind, dim, nc)
        rng = np.random.default_rng(7 + seed)
        JN = rng.normal(0, 1e-3, dim)
        rbb = rng.normal(0, 1, pt.nd)
        f = getattr(lib, f"bp_forward_{dim}_{nc}")
        r = getattr(lib, f"bp_reverse_{dim}_{nc}")

        def loss(I=pt.I, dI=pt.dI, ch=pt.ch):
            rb = np.zeros(pt.nd)
            f(ch, _ptr(pt.scal), _ptr(pt.uri), C.byref(bc), _ptr(I), _ptr(dI), _ptr(JN), _ptr(rb))
            loss.abs = float(np.abs(rbb * rb).sum())
            return float(rbb @ rb)

        Ib = np.zeros(pt.nd)
        dIb = np.zeros(dim * pt.nd)
        th = np.zeros(3 * nc)
        r(pt.ch, _ptr(pt.scal), _ptr(pt.uri), C.byref(bc), _ptr(pt.I), _ptr(pt.dI), _ptr(JN), _ptr(rbb),
          _ptr(Ib), _ptr(dIb), _ptr(th))
        for _ in range(3):
            dI_dir = rng.normal(0, 1, pt.dI.size) * np.abs(pt.dI)
            I_dir = rng.normal(0, 1, pt.nd) * np.maximum(np.abs(pt.I), 1e-3)
            h = 1e-6
            fd = (loss(pt.I + h * I_dir, pt.dI + h * dI_dir) - loss(pt.I - h * I_dir, pt.dI - h * dI_dir)) / (2 * h)
            an = float(Ib @ I_dir + dIb @ dI_dir)
            assert abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + 10 * 2.2e-16 * loss.abs / h, (seed, fd, an)
        loss()
        L_abs = loss.abs
        for c in range(nc):
            for k in range(3):
                an = th[3 * c + k] * pt.param_value(c, k)
                ok = []
                for h in (1e-2, 1e-3, 1e-4):
                    Lp = [loss(ch=pt.perturbed_chems(c, k, m * h)) for m in (1, -1, 2, -2)]
                    fd = (8 * (Lp[0] - Lp[1]) - (Lp[2] - Lp[3])) / (12 * h)
                    ok.append(abs(fd - an) <= 1e-5 * max(abs(fd), abs(an)) + 10 * 2.2e-16 * L_abs / h)
                assert any(ok), (seed, c, k, an)
