"""torch.autograd.Function over the assembled rhs, for tests only.

forward:  b = rhs(I; theta) through gales_asm_residual (FP64 form)
backward: (db/dI)^T g and (db/dtheta)^T g through gales_asm_vjp (mode EXACT)
theta is a (3*nb_comp,) tensor of the material parameters in the VJP's
parameterisation; the forward rebuilds the handle when theta changes.
"""
import importlib

import numpy as np
import torch

gm = importlib.import_module("gales-multi-fluid_gb300")
R_U = gm.R_UNIVERSAL


def material_from_theta(base: "gm.Material", theta: np.ndarray) -> "gm.Material":
    chems = []
    for c, q in enumerate(base.chemicals):
        t0, mu, cp = (float(v) for v in theta[3 * c:3 * c + 3])
        if q.kind == gm.abi.CH_CUSTOM:
            chems.append(gm.custom_chemical(rho=t0, mu=mu, cp=cp, kappa=q.kappa, alpha=q.alpha, beta=q.beta,
                                            chemical_diffusivity=q.chemical_diffusivity))
        else:
            chems.append(gm.ideal_gas_params(t0, mu, cp, q.kappa, chemical_diffusivity=q.chemical_diffusivity))
    return gm.Material(chems)


def theta_of(mat: "gm.Material") -> np.ndarray:
    out = []
    for q in mat.chemicals:
        out += [q.rho if q.kind == gm.abi.CH_CUSTOM else R_U / q.R, q.mu, q.cp]
    return np.array(out, dtype=np.float64)


class GalesRhs(torch.autograd.Function):
    @staticmethod
    def forward(ctx, I, theta, mesh, base_mat, setup, P, dt):
        mat = material_from_theta(base_mat, theta.detach().cpu().numpy())
        fa = gm.FluidAssembly(mesh, mat, setup)
        Id = I.detach().contiguous()
        b = torch.zeros_like(Id)
        fa.residual(Id, P, dt, b, form=gm.FORM_FP64)
        torch.cuda.synchronize()
        ctx.fa, ctx.P, ctx.dt = fa, P, dt
        ctx.save_for_backward(Id)
        return b

    @staticmethod
    def backward(ctx, g):
        (Id,) = ctx.saved_tensors
        fa = ctx.fa
        gI = torch.zeros_like(Id)
        gth = torch.zeros(3 * fa.nb_comp, dtype=torch.float64, device=Id.device)
        fa.vjp(Id, ctx.P, ctx.dt, g.contiguous(), gm.VJP_EXACT, gI, gth)
        torch.cuda.synchronize()
        return gI, gth, None, None, None, None, None
