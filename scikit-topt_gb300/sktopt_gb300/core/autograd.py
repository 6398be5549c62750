"""Differentiable compliance for PyTorch, with hand-written adjoint backward.

The density-method loop computes dC/drho by the chain
dC_drho_simp -> Heaviside derivative -> filter transpose
(sktopt/core/optimizers/common_density.py:1067-1101).  Here the same chain is
a composition of ``torch.autograd.Function`` objects whose backward passes
call the GPU kernels:

* ``GaussianFilterFn``: forward W rho (design rows), backward W^T g;
* ``HelmholtzFilterFn``: forward the nodal Helmholtz filter, backward its
  exact transpose (not the reference's clamped ``gradient``);
* ``ProjectionFn``: forward H(x), backward H'(x) g (projection.py:27-118);
* ``ComplianceFn``: forward solves K(rho) U = F and returns sum_j F_j . U_j
  (elasticity) or T^T K T (conduction); only U is saved, the element strains
  u_e^T K0 u_e are recomputed in backward, and the gradient is the
  self-adjoint one, -p (E0 - Emin) rho^(p-1) u_e^T K0 u_e per load case
  (derivatives.py:42-52).
"""
from __future__ import annotations

import numpy as np
import torch


class ComplianceFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, fem, p):
        rho = rho.detach().contiguous()
        L = fem.task.n_tasks
        U = torch.zeros((fem.task.n_dof, L), dtype=torch.float64, device=rho.device)
        comp = fem.solve_device(rho, p, U)
        ctx.fem, ctx.p = fem, p
        ctx.save_for_backward(rho, U)
        return torch.tensor(float(np.sum(comp)), dtype=torch.float64, device=rho.device)

    @staticmethod
    def backward(ctx, g):
        rho, U = ctx.saved_tensors
        _, dc = ctx.fem.sensitivity_multi_load(rho, ctx.p, U, dh=None, want_energy=False)
        return g * dc.sum(dim=1), None, None


class ProjectionFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, beta, eta):
        from .projection import heaviside_projection_device
        x = x.detach().contiguous()
        h, dh = torch.empty_like(x), torch.empty_like(x)
        heaviside_projection_device(x, beta, eta, out=h, dout=dh)
        ctx.save_for_backward(dh)
        return h

    @staticmethod
    def backward(ctx, g):
        (dh,) = ctx.saved_tensors
        return g * dh, None, None


class GaussianFilterFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, flt):
        ctx.flt = flt
        return flt.forward_device(x.detach().contiguous())

    @staticmethod
    def backward(ctx, g):
        return ctx.flt.gradient_device(g.contiguous()), None


class HelmholtzFilterFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, flt):
        ctx.flt = flt
        return flt.forward_device(x.detach().contiguous())

    @staticmethod
    def backward(ctx, g):
        return ctx.flt.vjp_device(g.contiguous()), None


def compliance(rho: torch.Tensor, fem, p: float = 3.0) -> torch.Tensor:
    """Compliance (sum over load cases) of the physical density ``rho``."""
    return ComplianceFn.apply(rho, fem, p)


def filtered_compliance(rho: torch.Tensor, fem, flt, p: float = 3.0, beta: float = 1.0,
                        eta: float = 0.5) -> torch.Tensor:
    """Compliance of H(F rho), F the Gaussian or the Helmholtz filter: the
    objective the OC loop differentiates."""
    Fn = HelmholtzFilterFn if hasattr(flt, "vjp_device") else GaussianFilterFn
    return ComplianceFn.apply(ProjectionFn.apply(Fn.apply(rho, flt), beta, eta), fem, p)
