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
that on ``torch.distributed`` (NCCL for CUDA tensors, gloo for host ones);
:func:`lsqr` does the same for LSQR.

The reference has no distributed code (PyLops runs one process); the
recurrences are those of ``pylops/optimization/cls_basic.py:334-708`` (CGLS)
and ``:711-1351`` (LSQR).
With two ranks the image sum is exact-order-independent (a + b = b + a); with
more, the order of the all-reduce is the backend's.
"""

from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from .linearoperator import LinearOperator
from .utils.backend import is_torch

__all__ = ["source_shard", "DistributedKirchhoff", "cgls", "lsqr"]


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


def _global_norm(a, group=None) -> float:
    return float(np.sqrt(_global_dot(a, a, group)))


def lsqr(Op: DistributedKirchhoff, y, x0: Optional = None, niter: int = 10, damp: float = 0.0, atol: float = 1e-8,
         btol: float = 1e-8, conlim: float = 1e8):
    """LSQR (``cls_basic.py:835-1136``) on a source-sharded operator: ``y`` is
    this rank's data, x0 and the result the (replicated) model.  The
    data-space vector u is sharded, so its norm is one float64 all-reduce per
    iteration; the model-space vectors v, w, x are the same on every rank and
    their norms are local.  Every scalar of the Golub-Kahan bidiagonalisation
    and the Paige-Saunders rotations is float64 and identical on all ranks.
    Returns ``(x, istop, iiter, r1norm, r2norm, anorm, acond, arnorm, xnorm,
    var, cost)`` as ``pylops.optimization.basic.lsqr`` (var is not computed:
    None)."""
    g = Op.group
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    dampsq = damp * damp
    anorm = acond = ddnorm = res2 = xnorm = xxnorm = z = 0.0
    cs2, sn2 = -1.0, 0.0
    if x0 is None:
        x = y.new_zeros(Op.shape[1]) if is_torch(y) else np.zeros(Op.shape[1], dtype=np.float64)
        u = y.clone() if is_torch(y) else np.array(y, dtype=np.float64, copy=True)
    else:
        x = x0.clone() if is_torch(x0) else np.array(x0, dtype=np.float64, copy=True)
        u = y - Op.matvec(x)
    alfa = 0.0
    beta = _global_norm(u, g)
    if beta > 0:
        u = u / beta
        v = Op.rmatvec(u)
        alfa = float(np.sqrt(abs(_local_dot(v, v))))
        if alfa > 0:
            v = v / alfa
    else:
        v = x.clone() if is_torch(x) else x.copy()
    w = v.clone() if is_torch(v) else v.copy()
    arnorm0 = alfa * beta
    rhobar, phibar, bnorm = alfa, beta, beta
    r1norm = r2norm = rnorm = beta
    arnorm = arnorm0
    cost = [beta]
    istop, iiter = 0, 0
    if arnorm0 == 0:
        return x, istop, iiter, r1norm, r2norm, anorm, acond, arnorm, xnorm, None, np.array(cost)
    while iiter < niter and istop == 0:
        # bidiagonalisation: u (sharded) and v (replicated)
        u = Op.matvec(v) - alfa * u
        beta = _global_norm(u, g)
        if beta > 0:
            u = u / beta
            anorm = float(np.sqrt(anorm ** 2 + alfa ** 2 + beta ** 2 + dampsq))
            v = Op.rmatvec(u) - beta * v
            alfa = float(np.sqrt(abs(_local_dot(v, v))))
            if alfa > 0:
                v = v / alfa
        # plane rotations (damping, then the bidiagonal)
        rhobar1 = float(np.hypot(rhobar, damp))
        cs1, sn1 = rhobar / rhobar1, damp / rhobar1
        psi = sn1 * phibar
        phibar = cs1 * phibar
        rho = float(np.hypot(rhobar1, beta))
        cs, sn = rhobar1 / rho, beta / rho
        theta = sn * alfa
        rhobar = -cs * alfa
        phi = cs * phibar
        phibar = sn * phibar
        tau = sn * phi
        t1, t2 = phi / rho, -theta / rho
        ddnorm += float(abs(_local_dot(w, w))) / (rho * rho)
        x = x + t1 * w
        w = v + t2 * w
        # norms and stopping tests (cls_basic.py:1066-1133)
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = float(np.sqrt(xxnorm + zbar ** 2))
        gamma = float(np.hypot(gambar, theta))
        cs2, sn2 = gambar / gamma, theta / gamma
        z = rhs / gamma
        xxnorm += z ** 2
        acond = anorm * float(np.sqrt(ddnorm))
        res2 += psi ** 2
        rnorm = float(np.sqrt(phibar ** 2 + res2))
        arnorm = alfa * abs(tau)
        r1sq = rnorm ** 2 - dampsq * xxnorm
        r1norm = float(np.sqrt(abs(r1sq))) * (-1.0 if r1sq < 0 else 1.0)
        r2norm = rnorm
        cost.append(abs(r1norm))
        test1 = rnorm / bnorm
        test2 = arnorm / arnorm0
        test3 = 1.0 / acond
        t1_ = test1 / (1.0 + anorm * xnorm / bnorm)
        rtol = btol + atol * anorm * xnorm / bnorm
        # the reference tests iiter before counting this iteration, so a run
        # that ends on niter leaves istop = 0 (cls_basic.py:1110-1136)
        if iiter >= niter:
            istop = 7
        if 1 + test3 <= 1:
            istop = 6
        if 1 + test2 <= 1:
            istop = 5
        if 1 + t1_ <= 1:
            istop = 4
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        iiter += 1
    return x, istop, iiter, r1norm, r2norm, anorm, acond, arnorm, xnorm, None, np.array(cost)
