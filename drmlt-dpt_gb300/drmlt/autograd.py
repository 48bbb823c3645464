"""torch.autograd view of the C-ABI derivative pair (check harness only).

`path_log_f(renderer, paths, u)` returns log f of each technique path at its
primary sample vector (drmlt_path_eval, the forward call); its gradient is the
gradient of drmlt_path_adjoint (the backward call: the reverse-mode adjoint),
and the gradient of that gradient (double backward, create_graph=True) is the
Hessian-vector product with the adjoint's forward-over-reverse Hessian -- the
PathFuncDerv pair of the reference's chad library (src/path.h:145-160) seen as
a differentiable function. The library computes
on the GPU from host arrays; tensors here live on the CPU.
"""
from __future__ import annotations

import numpy as np
import torch

from .capi import MAX_DIM


def _host(u: torch.Tensor) -> np.ndarray:
    a = np.zeros((u.shape[0], MAX_DIM), np.float32)
    a[:, :u.shape[1]] = u.detach().to("cpu", torch.float32).numpy()
    return a


class _PathGrad(torch.autograd.Function):
    """u -> gradient of log f (saved from the forward call); backward: H v."""

    @staticmethod
    def forward(ctx, u, grad, hess):
        ctx.save_for_backward(hess)
        return grad.clone()

    @staticmethod
    def backward(ctx, v):
        (hess,) = ctx.saved_tensors
        return torch.einsum("nij,nj->ni", hess, v), None, None


class _PathLogF(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, renderer, paths):
        d = u.shape[1]
        uh = _host(u)
        logf = renderer.path_eval(paths, uh)
        g, h = renderer.path_adjoint(paths, uh)
        grad = torch.from_numpy(np.ascontiguousarray(g[:, :d])).to(u.dtype)
        # each path's Hessian: d x d row-major at the start of its MAX_DIM^2 block
        hess = torch.from_numpy(np.ascontiguousarray(h.reshape(-1, MAX_DIM * MAX_DIM)[:, :d * d].reshape(-1, d, d)))
        hess = hess.to(u.dtype)
        ctx.save_for_backward(u, grad, hess)
        return torch.from_numpy(np.asarray(logf, np.float32)).to(u.dtype)

    @staticmethod
    def backward(ctx, go):
        u, grad, hess = ctx.saved_tensors
        return _PathGrad.apply(u, grad, hess) * go[:, None], None, None


def path_log_f(renderer, paths, u: torch.Tensor) -> torch.Tensor:
    """log f (n,) of n technique paths at u (n x dim, all paths of one dimension)."""
    return _PathLogF.apply(u, renderer, paths)
