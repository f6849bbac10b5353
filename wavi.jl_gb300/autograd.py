"""The velocity solve as a differentiable function of per-cell log C and log A (torch.autograd).

``VelocityFunction.apply(logC, logA, problem)`` returns the converged velocities (u, v), flattened in
column-major order from their reference shapes; ``backward`` is one ``wavi_adjoint_device`` call at the
forward solve's fixed point.  ``problem`` (a ``Problem``) holds a float64 ``VelocitySolver`` and a
``make_state(C, A)`` callable that returns (params, fields) for per-cell C and A arrays (built, for
example, with ``model.Model`` and ``pre_solve``).  The forward solve should be converged tightly: the
gradient is exact at the fixed point.
"""
import numpy as np
import torch


class Problem:
    """What VelocityFunction needs: the float64 solver, the state builder, the adjoint solve's settings."""

    def __init__(self, solver, make_state, tol=1e-10, maxiter=400):
        self.solver, self.make_state, self.tol, self.maxiter = solver, make_state, tol, maxiter


class VelocityFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, logC, logA, problem):
        g = problem.solver.grid
        shape = (g.nx, g.ny)
        C = np.exp(logC.detach().double().cpu().numpy().reshape(shape, order="F"))
        A = np.exp(logA.detach().double().cpu().numpy().reshape(shape, order="F"))
        params, fields = problem.make_state(C, A)
        ctx.stats = problem.solver.solve(params, fields)
        ctx.problem, ctx.params = problem, params
        dev = logC.device if logC.is_cuda else torch.device("cuda")
        u = torch.from_numpy(np.ascontiguousarray(fields["u"].ravel(order="F"))).to(dev)
        v = torch.from_numpy(np.ascontiguousarray(fields["v"].ravel(order="F"))).to(dev)
        return u, v

    @staticmethod
    def backward(ctx, gu, gv):
        p = ctx.problem
        g = p.solver.grid
        gc = torch.zeros(g.nx * g.ny, dtype=torch.float64, device="cuda")
        ga = torch.zeros_like(gc)
        p.solver.adjoint_device(ctx.params, gu.double().contiguous().cuda(), gv.double().contiguous().cuda(), gc, ga,
                                tol=p.tol, maxiter=p.maxiter)
        return gc, ga, None
