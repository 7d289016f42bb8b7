"""torch.autograd front end of the hand-written adjoint (gpmood_adj_* in libgpmood.so).

``FrozenMoodSteps.apply(u0, solver, nsteps, every)`` runs ``nsteps`` GP-MOOD
steps (the main.f90:145-203 loop: Setdt, SSP-RK3 with MOOD) from the padded
float64 CUDA tensor ``u0`` of shape (nf+8, lf+8, 4) and returns u_N.  Its
backward is the CUDA vector-Jacobian product of the same steps with every
step's MOOD order masks and dt frozen at their recorded values, recomputing
each segment of ``every`` steps from a checkpoint.  Gradients reach the
interior cells of u0 only (stage 1 refills the ghost cells by Boundary_C).

``frozen_replay(record, u0)`` re-applies a recording to another u0 (the map
whose Jacobian the backward transposes); it is differentiable the same way at
the recorded u0.
"""
from __future__ import annotations

import torch

from .gpmood import Adjoint, Solver


def _check_state(solver: Solver, u: torch.Tensor, name: str) -> torch.Tensor:
    if u.dtype != torch.float64 or not u.is_cuda or tuple(u.shape) != solver.shape:
        raise ValueError(f"{name} must be a CUDA float64 tensor of shape {solver.shape}")
    return u.contiguous()


class FrozenMoodSteps(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0: torch.Tensor, solver: Solver, nsteps: int, every: int = 10, t0: float = 0.0):
        u0 = _check_state(solver, u0, "u0")
        torch.cuda.current_stream().synchronize()
        solver.set_state_dev(u0.data_ptr(), t0)
        rec = solver.adj_record(nsteps, every)
        uN = torch.empty_like(u0)
        solver.get_state_dev(uN.data_ptr())
        ctx.record = rec
        return uN

    @staticmethod
    def backward(ctx, grad_uN: torch.Tensor):
        rec: Adjoint = ctx.record
        g = _check_state(rec.solver, grad_uN, "grad").detach()
        lam0 = torch.empty_like(g)
        torch.cuda.current_stream().synchronize()
        rec.backward(g.data_ptr(), lam0.data_ptr())
        return lam0, None, None, None, None


class _Replay(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0: torch.Tensor, rec: Adjoint):
        u0 = _check_state(rec.solver, u0, "u0")
        uN = torch.empty_like(u0)
        torch.cuda.current_stream().synchronize()
        rec.replay(u0.data_ptr(), uN.data_ptr())
        ctx.record = rec
        return uN

    @staticmethod
    def backward(ctx, grad_uN: torch.Tensor):
        rec: Adjoint = ctx.record
        g = _check_state(rec.solver, grad_uN, "grad").detach()
        lam0 = torch.empty_like(g)
        torch.cuda.current_stream().synchronize()
        rec.backward(g.data_ptr(), lam0.data_ptr())
        return lam0, None


def frozen_replay(rec: Adjoint, u0: torch.Tensor) -> torch.Tensor:
    return _Replay.apply(u0, rec)
