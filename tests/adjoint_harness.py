"""Check harness for the residual adjoint: the library's forward (residual)
and backward (transpose Jacobian-vector product) entry points wrapped in a
torch.autograd.Function, so torch's own gradient checker can drive them.
Test infrastructure only: the library itself has no torch dependency."""
import numpy as np
import torch


class ResidualFn(torch.autograd.Function):
    """R(q) of a FP64 solver (afx_residual) with its vJP (afx_residual_vjp)
    as the backward.  q: float64 tensor of 4*n_real entries, reference cell
    order."""

    @staticmethod
    def forward(ctx, q, solver):
        qn = q.detach().cpu().numpy().astype(np.float64)
        solver.set_q(qn)
        R = solver.residual()
        ctx.solver = solver
        ctx.save_for_backward(q.detach().clone())
        return torch.from_numpy(R).to(q.device)

    @staticmethod
    def backward(ctx, gR):
        (q,) = ctx.saved_tensors
        u, _ = ctx.solver.residual_vjp(gR.detach().cpu().numpy().astype(np.float64),
                                       q=q.cpu().numpy().astype(np.float64))
        return torch.from_numpy(u).to(gR.device), None
