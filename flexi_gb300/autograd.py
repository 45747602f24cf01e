"""torch.autograd bindings of the GPU right-hand side, the LSERK stepper and their adjoints.

For gradient checks and loss-driven studies: tensors are CPU float64 in the layout of U
(nElems, N+1, N+1, N+1, 5); the solver keeps its own device state. The backward passes call the
hand-written adjoint kernels through the C ABI (fg_vjp_time_derivative, fg_adjoint_forward/fg_adjoint_reverse);
nothing is differentiated by torch itself.
"""
import numpy as np
import torch

from .solver import Flexi


class TimeDerivative(torch.autograd.Function):
    """Ut = DGTimeDerivative_weakForm(U); backward: U_bar = (dUt/dU)^T Ut_bar."""

    @staticmethod
    def forward(ctx, U, solver: Flexi):
        solver.U = U.detach().cpu().numpy()
        Ut = solver.DGTimeDerivative_weakForm(0.0)
        ctx.solver = solver
        ctx.save_for_backward(U)
        return torch.from_numpy(Ut)

    @staticmethod
    def backward(ctx, gUt):
        (U,) = ctx.saved_tensors
        ctx.solver.U = U.detach().cpu().numpy()
        V, _ = ctx.solver.vjp_time_derivative(np.ascontiguousarray(gUt.detach().cpu().numpy()))
        return torch.from_numpy(V), None


class Solve(torch.autograd.Function):
    """U_T after n_steps LSERK steps of fixed dt from U0 with per-element viscosity multipliers mu_scale.

    backward returns the gradients with respect to U0 and mu_scale (checkpointed reverse sweep). The
    solver holds the checkpoints of its last forward, so call backward before the next Solve on it."""

    @staticmethod
    def forward(ctx, U0, mu_scale, solver: Flexi, n_steps: int, dt: float, ckpt_every: int):
        solver.U = U0.detach().cpu().numpy()
        solver.set_elem_mu_scale(mu_scale.detach().cpu().numpy())
        solver.adjoint_forward(n_steps, dt, ckpt_every)
        ctx.solver = solver
        return torch.from_numpy(solver.U)

    @staticmethod
    def backward(ctx, gUT):
        Ub0, mub = ctx.solver.adjoint_reverse(np.ascontiguousarray(gUT.detach().cpu().numpy()))
        return torch.from_numpy(Ub0), torch.from_numpy(mub), None, None, None, None


def kinetic_energy(U, weights_3d, jac):
    """Integrated kinetic energy sum_nodes w J |m|^2 / (2 rho) as a torch expression (weights_3d: (n,n,n)
    quadrature weights in (k, j, i) order, jac: (nElems, n, n, n) Jacobian determinant)."""
    rho = U[..., 0]
    m2 = U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2
    return (0.5 * m2 / rho * weights_3d * jac).sum()
