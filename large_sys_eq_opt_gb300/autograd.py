"""torch.autograd wrapper of the discrete adjoint, for checking gradients.

``FrozenSteps.apply(U0, solver, dts, ckpt_k)`` maps an initial Grid2D state
(torch float64, shape (ny+4, nx+4, 4), on the CPU) to the state after
len(dts) frozen-dt steps of ``solver`` (a large_sys_eq_opt_gb300.euler2d
Solver); its backward is eu_adjoint_backward.  The forward and adjoint run
on the GPU through the C ABI; torch only carries the tensors.
"""
from __future__ import annotations

import numpy as np
import torch


class FrozenSteps(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U0: torch.Tensor, solver, dts, ckpt_k: int = 32):
        solver.upload(U0.detach().cpu().numpy().astype(np.float64))
        solver.adjoint_forward(np.asarray(dts, dtype=np.float64), int(ckpt_k))
        ctx.solver = solver
        return torch.from_numpy(solver.download())

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        g = ctx.solver.adjoint_backward(grad_out.detach().cpu().numpy().astype(np.float64))
        return torch.from_numpy(g), None, None, None
