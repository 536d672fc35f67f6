"""Source-sharded Kirchhoff operator and CGLS across processes (one GPU each).

The operator shards naturally by source (each trace belongs to one
source-receiver pair): rank ``r`` of ``W`` builds the Kirchhoff operator of
its contiguous block of sources (:func:`source_shard`) and holds those
sources' traveltime/amplitude tables and data traces; every rank holds the
whole model (image points).  The forward needs no communication (each rank
produces its own traces); the adjoint sums the ranks' partial images with one
all-reduce; a solver needs global norms and dot products of data-space
vectors (one scalar all-reduce each), while model-space vectors are the same
on every rank.  :class:`DistributedKirchhoff` and :func:`cgls` implement
that on ``torch.distributed`` (NCCL for CUDA tensors, gloo for host ones).

The reference has no distributed code (PyLops runs one process); the
recurrences are those of ``pylops/optimization/cls_basic.py:334-708``.
With two ranks the image sum is exact-order-independent (a + b = b + a); with
more, the order of the all-reduce is the backend's.
"""

from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from .linearoperator import LinearOperator
from .utils.backend import is_torch

__all__ = ["source_shard", "DistributedKirchhoff", "cgls"]


def source_shard(ns: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous block [s0, s1) of the ns sources for ``rank`` of ``world``
    (the first ``ns % world`` ranks take one more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(ns, world)
    s0 = rank * base + min(rank, extra)
    return s0, s0 + base + (1 if rank < extra else 0)


def _allreduce(t, group=None):
    """In-place sum over ranks of a torch tensor, or of a numpy array (through
    a host tensor); returns the reduced array of the same kind."""
    import torch
    import torch.distributed as dist

    if is_torch(t):
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t
    tt = torch.from_numpy(np.ascontiguousarray(t))
    dist.all_reduce(tt, op=dist.ReduceOp.SUM, group=group)
    return tt.numpy()


def _local_dot(a, b) -> float:
    if is_torch(a):
        return float((a.double() * b.double()).sum())
    return float(np.dot(np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()))


def _global_dot(a, b, group=None) -> float:
    """Dot product of two data-space (sharded) vectors over all ranks."""
    import torch

    return float(_allreduce(torch.tensor([_local_dot(a, b)], dtype=torch.float64), group)[0])


class DistributedKirchhoff(LinearOperator):
    """This rank's rows of a source-sharded operator: ``local_op`` is the
    operator of this rank's sources (shape (traces of those sources x nt,
    ni)).  ``matvec`` returns this rank's data; ``rmatvec`` takes this rank's
    data and returns the full adjoint image (all ranks' partial images
    summed)."""

    def __init__(self, local_op: LinearOperator, group=None, name: str = "DK"):
        self.local = local_op
        self.group = group
        super().__init__(dtype=local_op.dtype, shape=local_op.shape, dims=local_op.dims, dimsd=local_op.dimsd,
                         name=name)

    def _matvec(self, x):
        return self.local.matvec(x)

    def _rmatvec(self, y):
        img = self.local.rmatvec(y)
        if is_torch(img):
            img = img.contiguous()
        else:
            img = np.array(img, copy=True)
        return _allreduce(img, self.group)


def cgls(Op: DistributedKirchhoff, y, x0: Optional = None, niter: int = 10, damp: float = 0.0, tol: float = 1e-4):
    """CGLS (``cls_basic.py:334-708``) on a source-sharded operator: ``y`` is
    this rank's data, x0 and the result are the (replicated) model.  Returns
    ``(x, istop, iiter, r1norm, r2norm, cost)`` as ``pylops.optimization.basic.cgls``
    (with the reference's ``r1norm = kold`` and its unsquared ``damp`` in the
    x0 set-up)."""
    g = Op.group
    dampsq = damp ** 2
    if x0 is None:
        x = (y.new_zeros(Op.shape[1]) if is_torch(y) else np.zeros(Op.shape[1], dtype=y.dtype))
        s = y.clone() if is_torch(y) else y.copy()
        c = Op.rmatvec(s)
    else:
        x = x0.clone() if is_torch(x0) else np.array(x0, copy=True)
        s = y - Op.matvec(x)
        c = Op.rmatvec(s) - damp * x
    q = Op.matvec(c)
    kold = abs(_local_dot(c, c))
    cost = [np.sqrt(_global_dot(s, s, g))]
    cost1 = [np.sqrt(cost[0] ** 2 + damp * abs(_local_dot(x, x)))]
    iiter = 0
    while iiter < niter and kold > tol:
        a = kold / (_global_dot(q, q, g) + dampsq * _local_dot(c, c))
        x = x + a * c
        s = s - a * q
        r = Op.rmatvec(s) - dampsq * x
        k = abs(_local_dot(r, r))
        b = k / kold
        c = r + b * c
        q = Op.matvec(c)
        kold = k
        iiter += 1
        cost.append(np.sqrt(_global_dot(s, s, g)))
        cost1.append(np.sqrt(cost[-1] ** 2 + dampsq * abs(_local_dot(x, x))))
    istop = 1 if kold < tol else 2
    return x, istop, iiter, kold, cost1[iiter], np.array(cost)
