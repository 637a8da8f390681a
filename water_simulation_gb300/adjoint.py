"""Differentiable DFSPH rollout for PyTorch.

The reference has no differentiable path. `Rollout` is a torch.autograd.Function
over the C ABI: its forward runs `n_steps` DFSPH steps on the GPU from (x0, v0)
with a checkpoint every `checkpoint_every` steps (dfsph_adjoint_forward), its
backward runs the hand-written adjoint kernels (dfsph_adjoint_backward), which
replay each segment once from its checkpoint, keep that segment's per-step
records (neighbour structure included) and differentiate it step by step in
reverse. Gradients come back for the initial positions, the initial
velocities and the XSPH coefficient (accumulated in FP64).

Tensors live on the solver's device in the solver's working type (float32, or
float64 for an FP64 context); every call goes through the solver on torch's
current stream, so no extra synchronisation is needed.
"""
from __future__ import annotations

import torch

from . import _lib
from .solver import Solver


def working_dtype(solver: Solver) -> torch.dtype:
    return torch.float64 if solver.config.precision == _lib.PRECISION_FP64 else torch.float32


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class Rollout(torch.autograd.Function):
    """(x0, v0, xsph) -> (x_T, v_T) after n_steps DFSPH steps."""

    @staticmethod
    def forward(ctx, x0, v0, xsph, solver: Solver, dt: float, n_steps: int, checkpoint_every: int):
        dtype = working_dtype(solver)
        for name, t in (("x0", x0), ("v0", v0)):
            if not t.is_cuda or t.dtype != dtype or t.dim() != 2 or t.shape[1] != 3:
                raise ValueError(f"{name} must be a CUDA tensor of shape (n, 3) and dtype {dtype}")
        n = x0.shape[0]
        if v0.shape[0] != n:
            raise ValueError("x0 and v0 differ in length")
        solver.set_stream(torch.cuda.current_stream(x0.device).cuda_stream)
        solver.set_xsph(float(xsph))
        x0c, v0c = x0.detach().contiguous(), v0.detach().contiguous()
        solver.adjoint_set_state_device(_ptr(x0c), _ptr(v0c), n)
        solver.adjoint_forward(dt, n_steps, checkpoint_every)
        xT = torch.empty_like(x0c)
        vT = torch.empty_like(v0c)
        solver.adjoint_state_device(_ptr(xT), _ptr(vT))
        ctx.solver = solver
        ctx.xsph_dtype = xsph.dtype if torch.is_tensor(xsph) else torch.float64
        ctx.xsph_device = xsph.device if torch.is_tensor(xsph) else torch.device("cpu")
        return xT, vT

    @staticmethod
    def backward(ctx, gx, gv):
        solver: Solver = ctx.solver
        ref = gx if gx is not None else gv
        gx = torch.zeros_like(ref) if gx is None else gx.contiguous()
        gv = None if gv is None else gv.contiguous()
        gx0 = torch.empty_like(gx)
        gv0 = torch.empty_like(gx)
        solver.set_stream(torch.cuda.current_stream(gx.device).cuda_stream)
        ge = solver.adjoint_backward_device(_ptr(gx), None if gv is None else _ptr(gv), _ptr(gx0), _ptr(gv0))
        g_eps = torch.tensor(ge, dtype=ctx.xsph_dtype, device=ctx.xsph_device)
        return gx0, gv0, g_eps, None, None, None, None


def rollout(solver: Solver, x0: torch.Tensor, v0: torch.Tensor, xsph, dt: float, n_steps: int,
            checkpoint_every: int = 20):
    """Differentiable (x_T, v_T); xsph may be a float or a 0-dim tensor."""
    if not torch.is_tensor(xsph):
        xsph = torch.tensor(float(xsph), dtype=torch.float64)
    return Rollout.apply(x0, v0, xsph, solver, dt, n_steps, checkpoint_every)


def drop_loss(x_T: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """mean over particles of |x_T - target|^2 (the differentiable-drop loss)."""
    return ((x_T - target) ** 2).sum(dim=1).mean()
