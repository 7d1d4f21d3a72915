"""torch.autograd interface of the split-step adjoint.

``split_step_objectives(solver, state0, ln_mult, t0, rho_u, ju, jb)`` runs
one split step of a flame batch on the GPU from ``state0`` with reaction-rate
multipliers exp(ln_mult) and returns the heat release rate Q_f and the
consumption speed S_c,f of every flame (FlameSolver::getHeatReleaseRate /
getConsumptionSpeed after the step). Its backward pass is the hand-written
discrete adjoint of the step (``ember_split_adjoint``): the forward step is
recomputed from the saved start state with a tape of the source stage (BDF
or QSS), and the gradients with respect to the start state and to ln(multiplier) of
every reaction are returned.
"""
from __future__ import annotations

import numpy as np
import torch


def _np(t):
    return np.ascontiguousarray(t.detach().cpu().numpy(), dtype=np.float64)


class SplitStepObjectives(torch.autograd.Function):
    """Inputs on a CUDA device stay there: the multipliers, the start state,
    the objectives and both gradients go through the library's device
    pointers without a host round trip; CPU tensors go through host arrays."""

    @staticmethod
    def forward(ctx, state0, ln_mult, solver, t0, rho_u, ju, jb, tape_cap):
        dev = state0.device if state0.is_cuda else None
        if dev is not None:
            solver.gmech.set_multipliers(torch.exp(ln_mult.detach().to(dev, torch.float64)).contiguous())
            solver.set_state(float(t0), state0.detach().to(torch.float64).contiguous())
            solver.step(1)
            _, hr, cs = solver.objectives(rho_u, ju, jb, device=dev)
            out = torch.cat([hr, cs])
        else:
            solver.gmech.set_multipliers(np.exp(_np(ln_mult)))
            solver.set_state(float(t0), _np(state0))
            solver.step(1)
            _, hr, cs = solver.objectives(rho_u, ju, jb)
            out = torch.as_tensor(np.concatenate([hr, cs]), dtype=torch.float64)
        ctx.solver, ctx.t0, ctx.rho_u, ctx.ju, ctx.jb, ctx.tape_cap = solver, t0, rho_u, ju, jb, tape_cap
        ctx.save_for_backward(state0, ln_mult)
        return out

    @staticmethod
    def backward(ctx, grad):
        state0, ln_mult = ctx.saved_tensors
        solver = ctx.solver
        nf = len(solver.grids)
        if state0.is_cuda:
            dev = state0.device
            g = grad.detach().to(dev, torch.float64).contiguous()
            solver.gmech.set_multipliers(torch.exp(ln_mult.detach().to(dev, torch.float64)).contiguous())
            solver.set_state(float(ctx.t0), state0.detach().to(torch.float64).contiguous())
            _, _, sbar, lbar = solver.adjoint(g[:nf], g[nf:], ctx.rho_u, ctx.ju, ctx.jb, ctx.tape_cap, device=dev)
            return (sbar.reshape(state0.shape), lbar.to(ln_mult.device), None, None, None, None, None, None)
        g = _np(grad)
        solver.gmech.set_multipliers(np.exp(_np(ln_mult)))
        solver.set_state(float(ctx.t0), _np(state0))
        _, _, sbar, lbar = solver.adjoint(g[:nf], g[nf:], ctx.rho_u, ctx.ju, ctx.jb, ctx.tape_cap)
        return (torch.as_tensor(sbar).reshape(state0.shape), torch.as_tensor(lbar), None, None, None, None, None,
                None)


def split_step_objectives(solver, state0, ln_mult, t0, rho_u, ju, jb, tape_cap: int = 0):
    """[Q_0..Q_{F-1}, S_c,0..S_c,F-1] after one split step, differentiable with
    respect to state0 [n_points, S+2] and ln_mult [n_reactions]."""
    return SplitStepObjectives.apply(state0, ln_mult, solver, t0, rho_u, ju, jb, tape_cap)
