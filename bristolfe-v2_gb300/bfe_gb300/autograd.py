"""torch.autograd view of the adjoint gradient (for checks against finite
differences and the FP64 adjoint; the computation is bfe_adjoint_gradient)."""
import numpy as np
import torch

from . import model
from .solver import VEL_CURRENT, Plan


class AscanMisfit(torch.autograd.Function):
    """J(s, rho) = 1/2 sum |A-scans(s, rho) - observed|^2.

    forward(s, rho, problem) with s, rho float64 CPU tensors of per-element
    stiffness scales and densities; problem = dict(element_data, n, dt, time,
    sources (1-based index lists), signal, monitors (1-based), observed,
    precision, gl_lookup). backward returns dJ/ds and dJ/drho from the
    adjoint march."""

    @staticmethod
    def forward(ctx, s, rho, problem):
        ke, mh, ch, dof = problem["element_data"]
        K, C, M = model.assemble_from_elements(ke, mh, ch, dof, problem["n"], s.numpy(), rho.numpy())
        with Plan(K, C, M, problem["dt"], VEL_CURRENT, problem.get("precision", "double"),
                  problem.get("gl_lookup")) as plan:
            # the gradient at (s, rho): scale the element data accordingly
            J, gs, gr = plan.adjoint_gradient(
                (ke * s.numpy()[:, None, None], mh * rho.numpy()[:, None], ch * rho.numpy()[:, None], dof),
                problem["time"], problem["sources"], problem["signal"], problem["monitors"],
                problem["observed"])
        # J is differentiated w.r.t. the scale of each element's data: convert
        # to d/ds and d/drho at the given point
        ctx.save_for_backward(torch.from_numpy(gs / s.numpy()), torch.from_numpy(gr / rho.numpy()))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        gs, gr = ctx.saved_tensors
        return grad_out * gs, grad_out * gr, None
