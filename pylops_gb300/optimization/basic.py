"""Functional solver entry points (``pylops/optimization/basic.py:90-332``)."""

from typing import Callable, Optional, Tuple

import numpy as np

from ..utils.backend import is_torch
from .cls_basic import CGLS, LSQR

__all__ = ["cgls", "lsqr"]


def _ravel_inputs(Op, y, x0):
    """``add_ndarray_support_to_solver`` (``pylops/utils/decorators.py:38-70``):
    flatten ndarray data/initial guess and remember to reshape the model."""
    reshape = None
    if y.ndim > 1 and tuple(y.shape) == tuple(getattr(Op, "dimsd", ())):
        y = y.reshape(-1)
        reshape = tuple(Op.dims)
    if x0 is not None and x0.ndim > 1:
        x0 = x0.reshape(-1)
        reshape = tuple(Op.dims)
    return y, x0, reshape


def cgls(Op, y, x0=None, niter: int = 10, damp: float = 0.0, tol: float = 1e-4, show: bool = False,
         itershow: Tuple[int, int, int] = (10, 10, 10), callback: Optional[Callable] = None,
         preallocate: bool = False):
    """Conjugate gradient least squares; returns
    ``(x, istop, iit, r1norm, r2norm, cost)`` like ``pylops.optimization.basic.cgls``."""
    y, x0, reshape = _ravel_inputs(Op, y, x0)
    solver = CGLS(Op)
    if callback is not None:
        solver.callback = callback
    x, istop, iiter, r1norm, r2norm, cost = solver.solve(y=y, x0=x0, tol=tol, niter=niter, damp=damp,
                                                         show=show, itershow=itershow, preallocate=preallocate)
    if reshape is not None:
        x = x.reshape(reshape)
    return x, istop, iiter, r1norm, r2norm, cost


def lsqr(Op, y, x0=None, damp: float = 0.0, atol: float = 1e-08, btol: float = 1e-08,
         conlim: float = 100000000.0, niter: int = 10, calc_var: bool = True, show: bool = False,
         itershow: Tuple[int, int, int] = (10, 10, 10), callback: Optional[Callable] = None,
         preallocate: bool = False):
    """LSQR; returns ``(x, istop, itn, r1norm, r2norm, anorm, acond, arnorm,
    xnorm, var, cost)`` like ``pylops.optimization.basic.lsqr``."""
    y, x0, reshape = _ravel_inputs(Op, y, x0)
    solver = LSQR(Op)
    if callback is not None:
        solver.callback = callback
    out = solver.solve(y=y, x0=x0, damp=damp, atol=atol, btol=btol, conlim=conlim, niter=niter,
                       calc_var=calc_var, show=show, itershow=itershow, preallocate=preallocate)
    x = out[0]
    if reshape is not None:
        x = x.reshape(reshape)
    return (x,) + tuple(out[1:])
