"""Wrap an operator into a torch autograd function
(``pylops/torchoperator.py:23-102``, ``pylops/_torchoperator.py``).

The forward pass applies ``Op`` and the backward pass its adjoint, so a
Kirchhoff operator (or any operator of this package) can sit inside a torch
model.  CUDA tensors are handed to the operator as they are -- the kernels
read and write torch's device memory on torch's current stream, no copy --
and CPU tensors go through numpy (the operator copies them to the device
inside the call).
"""

from __future__ import annotations

from typing import Optional

import numpy as np

from .linearoperator import LinearOperator

__all__ = ["TorchOperator"]


def _fn_class():
    import torch

    class _TorchOperator(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, forw, adj, device, devicetorch):
            ctx.forw, ctx.adj, ctx.device, ctx.devicetorch = forw, adj, device, devicetorch
            return _apply(forw, x, device, devicetorch)

        @staticmethod
        def backward(ctx, y):
            return _apply(ctx.adj, y, ctx.device, ctx.devicetorch), None, None, None, None

    return _TorchOperator


def _apply(fn, x, device, devicetorch):
    import torch

    if device == "gpu" or x.is_cuda:
        xx = x.detach()
        if not xx.is_cuda:
            xx = xx.cuda()
        y = fn(xx.contiguous())
        y = y if torch.is_tensor(y) else torch.as_tensor(np.asarray(y))
    else:
        y = torch.as_tensor(np.asarray(fn(x.detach().cpu().numpy())))
    return y.to(devicetorch)


class TorchOperator:
    """Torch function applying ``Op`` forward and ``Op.H`` backward.

    ``batch=True``: the input holds samples along its first axis.
    ``flatten``: samples are flattened (``True``) or shaped like ``Op.dims``.
    ``device``: ``'cpu'`` (numpy path) or ``'gpu'`` (device path; CUDA inputs
    always take it).  ``devicetorch``: device of the returned tensors."""

    def __init__(self, Op: LinearOperator, batch: bool = False, flatten: Optional[bool] = True,
                 device: str = "cpu", devicetorch: str = "cpu") -> None:
        self.device = device
        self.devicetorch = devicetorch
        self.dtype = np.dtype(Op.dtype)
        self.dims, self.dimsd = Op.dims, Op.dimsd
        self.name = Op.name
        self.transpf = tuple(np.roll(np.arange(2 if flatten else len(self.dims) + 1), -1))
        self.transpb = tuple(np.roll(np.arange(2 if flatten else len(self.dims) + 1), 1))
        if not batch:
            self.matvec = lambda x: Op @ x
            self.rmatvec = lambda x: Op.H @ x
        else:
            self.matvec = lambda x: _permute(Op @ _permute(x, self.transpf), self.transpb)
            self.rmatvec = lambda x: _permute(Op.H @ _permute(x, self.transpf), self.transpb)
        self.Top = _fn_class().apply

    def __call__(self, x):
        return self.apply(x)

    def apply(self, x):
        """Forward pass of ``x`` (torch tensor); differentiable."""
        return self.Top(x, self.matvec, self.rmatvec, self.device, self.devicetorch)


def _permute(x, order):
    import torch

    if torch.is_tensor(x):
        return x.permute(*order).contiguous()
    return np.ascontiguousarray(np.transpose(x, order))
