"""Batched least-squares migration: many independent Kirchhoff problems at once.

``KirchhoffBatch(ops)`` is the block-diagonal operator ``diag(K_1, ..., K_P)``
over the concatenated models and data of P kinematic
:class:`~pylops_gb300.waveeqprocessing.Kirchhoff` operators (any sizes).
Each application is a single launch per kernel over a work list covering all
problems, and :meth:`cgls` solves every problem with CGLS
(``pylops/optimization/cls_basic.py:334-708``) in one CUDA-graph launch with
per-problem float64 scalars and stopping rules.  In the reference the same
work is a Python loop over ``LSM`` problems.
"""

from __future__ import annotations

import ctypes
import time
from typing import List, Sequence

import numpy as np

from .. import _native
from ..linearoperator import LinearOperator
from ..utils.backend import is_torch
from .kirchhoff import Kirchhoff

__all__ = ["KirchhoffBatch"]


class KirchhoffBatch(LinearOperator):
    """Block-diagonal batch of kinematic Kirchhoff operators."""

    def __init__(self, ops: Sequence[Kirchhoff], dtype="float32", name: str = "KB"):
        ops = list(ops)
        if not ops:
            raise ValueError("empty batch")
        for k in ops:
            if not isinstance(k, Kirchhoff):
                raise TypeError("KirchhoffBatch takes Kirchhoff operators")
            if k.dynamic:
                raise NotImplementedError("the batch runs kinematic operators (dynamic=False)")
        self.ops = ops
        handles = (ctypes.c_void_p * len(ops))(*[k.native_handle.value for k in ops])
        h = ctypes.c_void_p()
        _native.check(_native.lib().kgb_batch_create(ctypes.byref(h), handles, len(ops)))
        self._h = h
        self.model_sizes = [k.shape[1] for k in ops]
        self.data_sizes = [k.shape[0] for k in ops]
        self.model_offsets = np.concatenate([[0], np.cumsum(self.model_sizes)])
        self.data_offsets = np.concatenate([[0], np.cumsum(self.data_sizes)])
        super().__init__(dtype=np.dtype(dtype), shape=(int(self.data_offsets[-1]), int(self.model_offsets[-1])),
                         name=name)
        self.tile = 8
        self.gather_shape = (8, 1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _native._lib is not None:
            try:
                _native._lib.kgb_batch_destroy(h)
            except Exception:  # pragma: no cover
                pass
            self._h = None

    # ------------------------------------------------------------ apply
    def _apply(self, x, forward: bool):
        import torch

        n_out = self.shape[0] if forward else self.shape[1]
        xx = x.to(device="cuda", dtype=torch.float32).contiguous() if is_torch(x) else \
            torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device="cuda")
        y = torch.empty(n_out, dtype=torch.float32, device="cuda")
        fn = _native.lib().kgb_batch_forward if forward else _native.lib().kgb_batch_adjoint
        _native.check(fn(self._h, xx.data_ptr(), y.data_ptr(), torch.cuda.current_stream().cuda_stream))
        if is_torch(x):
            return y
        return y.cpu().numpy().astype(self.dtype, copy=False)

    def _matvec(self, x):
        return self._apply(x, True)

    def _rmatvec(self, x):
        return self._apply(x, False)

    def split_model(self, x) -> List:
        """Per-problem pieces of a concatenated model vector."""
        return [x[self.model_offsets[p]:self.model_offsets[p + 1]] for p in range(len(self.ops))]

    def split_data(self, d) -> List:
        return [d[self.data_offsets[p]:self.data_offsets[p + 1]] for p in range(len(self.ops))]

    # ------------------------------------------------------------ tuning
    def set_tile(self, receivers_per_item: int) -> None:
        _native.check(_native.lib().kgb_batch_set_tile(self._h, int(receivers_per_item)))
        self.tile = int(receivers_per_item)

    def set_gather(self, receivers_in_registers: int, points_per_thread: int) -> None:
        _native.check(_native.lib().kgb_batch_set_gather(self._h, int(receivers_in_registers),
                                                         int(points_per_thread)))
        self.gather_shape = (int(receivers_in_registers), int(points_per_thread))

    def autotune(self, candidates=(2, 4, 8), gather_candidates=((4, 1), (8, 1), (4, 2), (8, 2)),
                 reps: int = 3) -> dict:
        """Time the forward for each forward tile (receivers per work item)
        and the adjoint for each gather shape (receivers in registers, image
        points per thread) on this batch, keep the fastest of each and
        return the timings ({R: ms} for the forward, {"gather rc x ppt": ms}
        for the adjoint).  Every choice is deterministic; the forward tile and
        the receivers held in registers group the sums differently, so the
        results agree to float32 rounding."""
        import torch

        m = torch.randn(self.shape[1], device="cuda")
        d = torch.empty(self.shape[0], device="cuda")
        stream = torch.cuda.current_stream()
        L = _native.lib()
        times = {}
        for R in candidates:
            self.set_tile(R)
            _native.check(L.kgb_batch_forward(self._h, m.data_ptr(), d.data_ptr(), stream.cuda_stream))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                _native.check(L.kgb_batch_forward(self._h, m.data_ptr(), d.data_ptr(), stream.cuda_stream))
            e1.record(stream)
            torch.cuda.synchronize()
            times[R] = e0.elapsed_time(e1) / reps
        best = min(times, key=times.get)
        self.set_tile(best)
        gtimes = {}
        for rc, ppt in gather_candidates:
            self.set_gather(rc, ppt)
            _native.check(L.kgb_batch_adjoint(self._h, d.data_ptr(), m.data_ptr(), stream.cuda_stream))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                _native.check(L.kgb_batch_adjoint(self._h, d.data_ptr(), m.data_ptr(), stream.cuda_stream))
            e1.record(stream)
            torch.cuda.synchronize()
            gtimes[(rc, ppt)] = e0.elapsed_time(e1) / reps
        gbest = min(gtimes, key=gtimes.get)
        self.set_gather(*gbest)
        times.update({f"gather {rc}x{ppt}": t for (rc, ppt), t in gtimes.items()})
        return times

    # ------------------------------------------------------------ solver
    def cgls(self, y, niter: int = 20, damp: float = 0.0, tol: float = 1e-4, use_graph: bool = True):
        """CGLS on every problem (x0 = 0).  Returns ``(x, iiter, kold, cost)``:
        the concatenated model (kind of ``y``), per-problem iteration counts,
        final ``kold`` (the reference's ``r1norm``) and residual histories
        (P x (niter+1))."""
        import torch

        yy = y.to(device="cuda", dtype=torch.float32).contiguous() if is_torch(y) else \
            torch.as_tensor(np.ascontiguousarray(y, dtype=np.float32), device="cuda")
        x = torch.empty(self.shape[1], dtype=torch.float32, device="cuda")
        P = len(self.ops)
        cost = np.zeros((P, niter + 1))
        iiter = np.zeros(P, dtype=np.int32)
        kold = np.zeros(P)
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            _native.check(_native.lib().kgb_batch_cgls(
                self._h, yy.data_ptr(), x.data_ptr(), int(niter), float(damp), float(tol), int(bool(use_graph)),
                _native.dptr(cost), _native.iptr(iiter), _native.dptr(kold), stream.cuda_stream))
        torch.cuda.current_stream().wait_stream(stream)
        xout = x if is_torch(y) else x.cpu().numpy()
        return xout, iiter, kold, cost


def random_problems(n: int, seed: int = 0, nt: int = 501, dt: float = 0.004, f0: float = 25.0):
    """Seeded batch of the batched-LSM workload: per problem a constant
    velocity U[1500, 3500] m/s, nz in U[64, 200], nx in U[64, 256] at 4 m,
    8-32 sources and 32-128 receivers at the surface, a 25 Hz Ricker, and a
    reflectivity of 2-6 random-dip layers.  Returns a list of dicts with the
    Kirchhoff arguments and the true reflectivity."""
    from ..utils.wavelets import ricker

    rng = np.random.default_rng(seed)
    t = np.arange(nt) * dt
    wav, _, wc = ricker(t[:41], f0=f0)
    out = []
    for _ in range(n):
        nz, nx = int(rng.integers(64, 201)), int(rng.integers(64, 257))
        ns, nr = int(rng.integers(8, 33)), int(rng.integers(32, 129))
        vel = float(rng.uniform(1500.0, 3500.0))
        z = np.arange(nz) * 4.0
        x = np.arange(nx) * 4.0
        srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
        recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
        refl = np.zeros((nx, nz))
        for _ in range(int(rng.integers(2, 7))):
            z0 = rng.uniform(8, nz - 8)
            dip = np.tan(np.deg2rad(rng.uniform(-20, 20)))
            a = rng.standard_normal()
            iz = np.round(z0 + dip * (np.arange(nx) - nx / 2)).astype(int)
            ok = (iz >= 0) & (iz < nz)
            refl[np.arange(nx)[ok], iz[ok]] += a
        out.append(dict(z=z, x=x, t=t, srcs=srcs, recs=recs, vel=vel, wav=wav, wavcenter=wc, refl=refl))
    return out


def build_batch(problems, dtype="float32"):
    """Kirchhoff operators (analytic, kinematic) for ``random_problems`` output."""
    ops = [Kirchhoff(p["z"], p["x"], p["t"], p["srcs"], p["recs"], p["vel"], p["wav"], p["wavcenter"],
                     mode="analytic", dynamic=False, dtype=dtype) for p in problems]
    return KirchhoffBatch(ops, dtype=dtype)
