"""torch.autograd harness around the C-ABI solve and its hand-written adjoint.

    x = SparseSolve.apply(vals, b, A, ctx, rtol)

solves A(vals) x = b with hhp_bicgstab_dev and, on backward, calls hhp_bicgstab_backward_dev:
lambda = A^-T dL/dx (BiCGStab on the device-built transpose), dL/db = lambda and
dL/dvals_k = -lambda[row(k)] * x[col(k)] for every stored entry k of A. Torch only carries the
tensors and the graph; both directions run in libhhp_gpu.so.
"""
from __future__ import annotations

import torch

from .api import Context, Matrix, bicgstab, bicgstab_backward


class SparseSolve(torch.autograd.Function):
    @staticmethod
    def forward(fctx, vals: torch.Tensor, b: torch.Tensor, A: Matrix, ctx: Context, rtol: float = 1e-12,
                maxit: int = 20000, precision: str = "fp64"):
        vals_c = vals.detach().contiguous()
        A.set_values(vals_c)
        torch.cuda.synchronize()
        x = torch.zeros_like(b)
        x, res = bicgstab(ctx, A, b.detach().contiguous(), x, rtol=rtol, maxit=maxit, precision=precision)
        fctx.A, fctx.ctx, fctx.rtol, fctx.maxit, fctx.precision = A, ctx, rtol, maxit, precision
        fctx.save_for_backward(x)
        return x

    @staticmethod
    def backward(fctx, grad_x: torch.Tensor):
        (x,) = fctx.saved_tensors
        dldb, dlda, _ = bicgstab_backward(fctx.ctx, fctx.A, x, grad_x.contiguous(), rtol=fctx.rtol,
                                          maxit=fctx.maxit, precision=fctx.precision,
                                          want_dlda=fctx.needs_input_grad[0])
        return dlda, dldb, None, None, None, None, None
