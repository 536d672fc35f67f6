"""CGLS and LSQR solvers (``pylops/optimization/cls_basic.py:334-1351``).

Two execution paths, same API and arithmetic as the reference classes:

* **device-resident** (operator is a :class:`~pylops_gb300.waveeqprocessing.Kirchhoff`):
  the vectors stay in HBM as float32, every dot product, norm and scalar
  recurrence is float64 on the GPU (``kgb_solver_*`` in the C ABI), and
  ``run`` replays one captured iteration inside a CUDA-graph WHILE node
  whose condition is the reference's stopping test -- one graph launch per
  ``run`` and no host synchronisation between iterations;
* **generic** (any other :class:`~pylops_gb300.LinearOperator`, e.g. a
  preconditioned product ``Op @ P``): the reference's recurrences on numpy
  or torch vectors with float64 scalars.
"""

from __future__ import annotations

import ctypes
import time
from typing import Optional, Tuple

import numpy as np

from .. import _native
from ..utils.backend import is_torch, to_numpy
from .basesolver import Solver, _units

__all__ = ["CGLS", "LSQR"]


# ----------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------
def _device_parts(Op):
    """(Kirchhoff, right diagonal or None) when the solve can run on the
    device path: a Kirchhoff operator, or ``Kop * Diagonal(p)`` with a real
    diagonal (a right preconditioner); None otherwise."""
    from ..basicoperators.diagonal import Diagonal
    from ..linearoperator import _ProductLinearOperator
    from ..waveeqprocessing.kirchhoff import Kirchhoff

    if isinstance(Op, Kirchhoff):
        return Op, None
    if isinstance(Op, _ProductLinearOperator):
        A, B = Op.args
        if isinstance(A, Kirchhoff) and isinstance(B, Diagonal) and not B.complex:
            d = B.diag.detach().cpu().numpy() if is_torch(B.diag) else np.asarray(B.diag)
            if B._bshape is not None:
                d = np.broadcast_to(d.reshape(B._bshape), B.dims)
            return A, np.ascontiguousarray(d, dtype=np.float32).reshape(-1)
    return None


def _is_device_kirchhoff(Op) -> bool:
    return _device_parts(Op) is not None


def _dot(a, b) -> float:
    """float64 inner product of two real vectors."""
    if is_torch(a):
        import torch

        if a.is_cuda and a.dtype == torch.float32 and b.dtype == torch.float32:
            out = torch.empty(1, dtype=torch.float64, device=a.device)
            _native.check(_native.lib().kgb_dot_f64(a.contiguous().data_ptr(), b.contiguous().data_ptr(),
                                                    a.numel(), out.data_ptr(),
                                                    torch.cuda.current_stream().cuda_stream))
            return float(out.item())
        return float(torch.dot(a.double().reshape(-1), b.double().reshape(-1)).item())
    return float(np.dot(np.asarray(a, dtype=np.float64).ravel(), np.asarray(b, dtype=np.float64).ravel()))


def _norm(a) -> float:
    return float(np.sqrt(_dot(a, a)))


def _copy(a):
    return a.clone() if is_torch(a) else a.copy()


def _zeros_like_model(Op, y):
    if is_torch(y):
        import torch

        return torch.zeros(Op.shape[1], dtype=y.dtype, device=y.device)
    return np.zeros(Op.shape[1], dtype=y.dtype)


class _DeviceSolver:
    """Owner of a ``kgb_solver`` handle and of the stream it runs on."""

    def __init__(self, Op, kind: int):
        import torch

        self.torch = torch
        self.Op = Op
        self.kind = kind
        self.stream = torch.cuda.Stream()
        kop, diag = _device_parts(Op)
        h = ctypes.c_void_p()
        _native.check(_native.lib().kgb_solver_create(ctypes.byref(h), kop.native_handle, kind))
        self.h = h
        self.diag = None
        if diag is not None:
            self.diag = torch.as_tensor(diag, device="cuda")
            _native.check(_native.lib().kgb_solver_set_diagonal(h, self.diag.data_ptr()))
        self.out = np.zeros(16)

    def __del__(self):
        if getattr(self, "h", None) is not None and _native._lib is not None:
            try:
                self.stream.synchronize()
                _native._lib.kgb_solver_destroy(self.h)
            except Exception:  # pragma: no cover
                pass
            self.h = None

    def _dev(self, v):
        torch = self.torch
        if v is None:
            return None
        return torch.as_tensor(v if is_torch(v) else np.ascontiguousarray(v, dtype=np.float32),
                               device="cuda").to(torch.float32).contiguous()

    def setup(self, y, x0, params):
        torch = self.torch
        cur = torch.cuda.current_stream()
        self.stream.wait_stream(cur)
        self.y = self._dev(y)
        self.x0 = self._dev(x0)
        p = np.ascontiguousarray(params, dtype=np.float64)
        with torch.cuda.stream(self.stream):
            _native.check(_native.lib().kgb_solver_setup(
                self.h, self.y.data_ptr(), 0 if self.x0 is None else self.x0.data_ptr(), _native.dptr(p),
                len(p), self.stream.cuda_stream))

    def run(self, niter: int, graph: bool):
        with self.torch.cuda.stream(self.stream):
            _native.check(_native.lib().kgb_solver_run(self.h, int(niter), int(bool(graph)), self.stream.cuda_stream))

    def result(self, want_x=True, cost_cap=0):
        torch = self.torch
        x = torch.empty(self.Op.shape[1], dtype=torch.float32, device="cuda") if want_x else None
        cost = np.zeros(max(cost_cap, 1))
        _native.check(_native.lib().kgb_solver_result(
            self.h, 0 if x is None else x.data_ptr(), _native.dptr(self.out), _native.dptr(cost), int(cost_cap),
            self.stream.cuda_stream))
        torch.cuda.current_stream().wait_stream(self.stream)
        return x, self.out.copy(), cost


def _has_user_callback(solver) -> bool:
    """True when a per-iteration ``callback`` was attached to the instance or
    overridden in a subclass (the solve then steps from the host)."""
    return "callback" in solver.__dict__ or type(solver).callback is not Solver.callback


def _like_input(x_dev, ref):
    """Return a device result in the kind (numpy/torch) and dtype of the user's data."""
    if is_torch(ref):
        return x_dev if x_dev.dtype == ref.dtype else x_dev.to(ref.dtype)
    return x_dev.cpu().numpy().astype(ref.dtype, copy=False)


# ----------------------------------------------------------------------------
# CGLS
# ----------------------------------------------------------------------------
class CGLS(Solver):
    r"""Conjugate gradient least squares (``cls_basic.py:334-708``).

    Minimises :math:`\|y - Op\,x\|_2^2 + \epsilon^2 \|x\|_2^2`.
    """

    def _print_setup(self, xcomplex: bool = False) -> None:
        self._print_solver(nbar=65)
        if self.niter is not None:
            print(f"damp = {self.damp:10e}\ttol = {self.tol:10e}\tniter = {self.niter}")
        else:
            print(f"damp = {self.damp:10e}\ttol = {self.tol:10e}\t")
        print("-" * 65 + "\n")
        print("    Itn          x[0]              r1norm         r2norm")

    def _print_step(self, x) -> None:
        x0 = float(to_numpy(x[:1])[0])
        print(f"{self.iiter:6g}       {x0:11.4e}        {self.cost[self.iiter]:11.4e}    {self.cost1[self.iiter]:11.4e}")

    def memory_usage(self, show: bool = False, unit: str = "B") -> float:
        nbytes = 4 if _is_device_kirchhoff(self.Op) else np.dtype(self.Op.dtype).itemsize
        memuse = (2 * self.Op.shape[1] + 3 * self.Op.shape[0]) * nbytes + (3 * self.Op.shape[1]) * nbytes
        if show:
            print(f"CGLS predicted memory usage: {memuse / _units[unit]:.2f} {unit}")
        return memuse

    def setup(self, y, x0=None, niter: Optional[int] = None, damp: float = 0.0, tol: float = 1e-4,
              preallocate: bool = False, show: bool = False):
        """Setup (``cls_basic.py:432-506``)."""
        self.y = y
        self.damp = damp ** 2
        self.tol = tol
        self.niter = niter
        self.preallocate = preallocate
        self._ydtype = y.dtype
        self._native = _is_device_kirchhoff(self.Op)
        if self._native:
            self._dev = _DeviceSolver(self.Op, 0)
            self._dev.setup(y, x0, [damp, tol])
            x_dev, out, cost = self._dev.result(want_x=True, cost_cap=2)
            self.kold = float(out[9])
            self.cost = [float(cost[0])]
            self.cost1 = [float(cost[1])]
            self.iiter = 0
            x = _like_input(x_dev, y)
        else:
            if x0 is None:
                x = _zeros_like_model(self.Op, y)
                self.s = _copy(y)
                self.c = self.Op.rmatvec(self.s)
            else:
                x = _copy(x0)
                self.s = y - self.Op.matvec(x)
                self.c = self.Op.rmatvec(self.s) - damp * x
            self.q = self.Op.matvec(self.c)
            self.kold = abs(_dot(self.c, self.c))
            self.cost = [_norm(self.s)]
            self.cost1 = [float(np.sqrt(self.cost[0] ** 2 + damp * abs(_dot(x, x))))]
            self.iiter = 0
        if show:
            self._print_setup()
        return x

    def _sync_native(self, want_x=True):
        _, out, _ = self._dev.result(want_x=False, cost_cap=0)
        n = int(out[0]) + 1
        x_dev, out, cost = self._dev.result(want_x=want_x, cost_cap=2 * n)
        self.iiter = int(out[0])
        self.kold = float(out[9])
        self.cost = list(cost[:n])
        self.cost1 = list(cost[n:2 * n])
        return x_dev

    def step(self, x, show: bool = False):
        """One iteration (``cls_basic.py:508-568``)."""
        if self._native:
            self._dev.run(1, graph=False)
            x_dev = self._sync_native()
            x = _like_input(x_dev, self.y)
        else:
            a = self.kold / (_dot(self.q, self.q) + self.damp * _dot(self.c, self.c))
            x = x + a * self.c
            self.s = self.s - a * self.q
            r = self.Op.rmatvec(self.s) - self.damp * x
            k = abs(_dot(r, r))
            b = k / self.kold
            self.c = r + b * self.c
            self.q = self.Op.matvec(self.c)
            self.kold = k
            self.iiter += 1
            self.cost.append(_norm(self.s))
            self.cost1.append(float(np.sqrt(self.cost[self.iiter] ** 2 + self.damp * abs(_dot(x, x)))))
        if show:
            self._print_step(x)
        return x

    def run(self, x, niter: Optional[int] = None, show: bool = False, itershow=(10, 10, 10)):
        """Iterate while ``iiter < niter and kold > tol`` (``cls_basic.py:570-608``)."""
        niter = self.niter if niter is None else niter
        if niter is None:
            raise ValueError("niter must not be None")
        if self._native and not show and not self.callbacks and not _has_user_callback(self):
            self._dev.run(niter - self.iiter, graph=True)
            x_dev = self._sync_native()
            return _like_input(x_dev, self.y)
        while self.iiter < niter and self.kold > self.tol:
            showstep = show and (self.iiter < itershow[0] or niter - self.iiter < itershow[1]
                                 or self.iiter % itershow[2] == 0)
            x = self.step(x, showstep)
            self.callback(x)
        return x

    def finalize(self, show: bool = False) -> None:
        """``cls_basic.py:610-631``: istop, r1norm (= kold, as the reference), r2norm."""
        self.tend = time.time()
        self.telapsed = self.tend - self.tstart
        self.istop = 1 if self.kold < self.tol else 2
        self.r1norm = self.kold
        self.r2norm = self.cost1[self.iiter]
        if show:
            self._print_finalize(nbar=65)
        self.cost = np.array(self.cost)

    def solve(self, y, x0=None, niter: int = 10, damp: float = 0.0, tol: float = 1e-4,
              preallocate: bool = False, show: bool = False, itershow=(10, 10, 10)):
        x = self.setup(y=y, x0=x0, niter=niter, damp=damp, tol=tol, preallocate=preallocate, show=show)
        x = self.run(x, niter, show=show, itershow=itershow)
        self.finalize(show)
        return x, self.istop, self.iiter, self.r1norm, self.r2norm, self.cost


# ----------------------------------------------------------------------------
# LSQR
# ----------------------------------------------------------------------------
class LSQR(Solver):
    r"""LSQR (Paige & Saunders 1982), ``cls_basic.py:711-1351``."""

    def __init__(self, Op, callbacks=None):
        super().__init__(Op, callbacks)
        self.msg = (
            "The exact solution is x = 0                               ",
            "Op x - b is small enough, given atol, btol                 ",
            "The least-squares solution is good enough, given atol     ",
            "The estimate of cond(Opbar) has exceeded conlim            ",
            "Op x - b is small enough for this machine                  ",
            "The least-squares solution is good enough for this machine",
            "Cond(Opbar) seems to be too large for this machine         ",
            "The iteration limit has been reached                      ",
        )

    def _print_setup(self, x, xcomplex: bool = False) -> None:
        self._print_solver(nbar=90)
        print(f"damp = {self.damp:20.14e}     calc_var = {self.calc_var:6g}")
        print(f"atol = {self.atol:8.2e}                 conlim = {self.conlim:8.2e}")
        print(f"btol = {self.btol:8.2e}                 niter = {self.niter:8g}")
        print("-" * 90)
        print("   Itn     x[0]      r1norm     r2norm   Compatible   LS     Norm A   Cond A")
        x0 = float(to_numpy(x[:1])[0])
        test2 = self.alfa / self.beta if self.beta else 0.0
        print(f"{0:6g} {x0:11.4e} {self.r1norm:10.3e} {self.r2norm:10.3e}  {1:8.1e} {test2:8.1e}")

    def _print_step(self, x) -> None:
        x0 = float(to_numpy(x[:1])[0])
        print(f"{self.iiter:6g} {x0:11.4e} {self.r1norm:10.3e} {self.r2norm:10.3e}  "
              f"{self.test1:8.1e} {self.test2:8.1e} {self.anorm:8.1e} {self.acond:8.1e}")

    def _print_finalize(self) -> None:
        print(" ")
        print(f"LSQR finished, {self.msg[self.istop]}")
        print(" ")
        print(f"istop ={self.istop:8g}   r1norm ={self.r1norm:8.1e}   anorm ={self.anorm:8.1e}   arnorm ={self.arnorm:8.1e}")
        print(f"itn   ={self.iiter:8g}   r2norm ={self.r2norm:8.1e}   acond ={self.acond:8.1e}   xnorm  ={self.xnorm:8.1e}")
        print(f"Total time (s) = {self.telapsed:.2f}")
        print("-" * 90 + "\n")

    def memory_usage(self, show: bool = False, unit: str = "B") -> float:
        nbytes = 4 if _is_device_kirchhoff(self.Op) else np.dtype(self.Op.dtype).itemsize
        memuse = (4 * self.Op.shape[1] + 2 * self.Op.shape[0]) * nbytes + self.Op.shape[1] * nbytes
        if show:
            print(f"LSQR predicted memory usage: {memuse / _units[unit]:.2f} {unit}")
        return memuse

    def setup(self, y, x0=None, damp: float = 0.0, atol: float = 1e-08, btol: float = 1e-08,
              conlim: float = 100000000.0, niter: int = 10, calc_var: bool = True,
              preallocate: bool = False, show: bool = False):
        """Setup (``cls_basic.py:835-985``)."""
        self.y = y
        self.damp = damp
        self.atol = atol
        self.btol = btol
        self.conlim = conlim
        self.niter = niter
        self.calc_var = calc_var
        self.preallocate = preallocate
        self._ydtype = y.dtype
        self.iiter = 0
        self.istop = 0
        self.ctol = 1.0 / conlim if conlim > 0 else 0
        self._native = _is_device_kirchhoff(self.Op)
        if self._native:
            self._dev = _DeviceSolver(self.Op, 1)
            self._dev.setup(y, x0, [damp, atol, btol, conlim, niter])
            x_dev, out, cost = self._dev.result(want_x=True, cost_cap=1)
            self._read_state(out, cost)
            x = _like_input(x_dev, y)
            self.alfa = self.arnorm / self.beta if self.beta else 0.0
        else:
            self.var = None
            self.var_scalar = 0.0
            self.anorm = 0.0
            self.acond = 0.0
            self.dampsq = damp ** 2
            self.ddnorm = 0.0
            self.res2 = 0.0
            self.xnorm = 0.0
            self.xxnorm = 0.0
            self.z = 0.0
            self.cs2 = -1.0
            self.sn2 = 0.0
            if x0 is None:
                x = _zeros_like_model(self.Op, y)
                self.u = _copy(y)
            else:
                x = _copy(x0)
                self.u = y - self.Op.matvec(x0)
            self.alfa = 0.0
            self.beta = _norm(self.u)
            if self.beta > 0.0:
                self.u = self.u / self.beta
                self.v = self.Op.rmatvec(self.u)
                self.alfa = _norm(self.v)
                if self.alfa > 0:
                    self.v = self.v / self.alfa
            else:
                self.v = _copy(x)
                self.alfa = 0
            self.w = _copy(self.v)
            self.arnorm = self.alfa * self.beta
            self.arnorm0 = self.arnorm
            self.rhobar = self.alfa
            self.phibar = self.beta
            self.bnorm = self.beta
            self.rnorm = self.beta
            self.r1norm = self.rnorm
            self.r2norm = self.rnorm
            self.cost = [float(self.rnorm)]
        self.test1 = 1.0
        self.test2 = 0.0
        self.test3 = 0.0
        if show:
            self._print_setup(x)
        return x

    def _read_state(self, out, cost):
        n = int(out[0])
        self.iiter = n
        self.istop = int(out[1])
        self.r1norm, self.r2norm, self.anorm, self.acond = float(out[2]), float(out[3]), float(out[4]), float(out[5])
        self.arnorm, self.xnorm, self.var_scalar = float(out[6]), float(out[7]), float(out[8])
        self.cost = list(cost[: n + 1])
        self.bnorm = float(self.cost[0])
        self.beta = self.bnorm if n == 0 else getattr(self, "beta", self.bnorm)
        self.rnorm = self.r2norm
        self.test1 = self.rnorm / self.bnorm if self.bnorm else 0.0

    def _sync_native(self, want_x=True):
        _, out, _ = self._dev.result(want_x=False, cost_cap=0)
        x_dev, out, cost = self._dev.result(want_x=want_x, cost_cap=int(out[0]) + 1)
        self._read_state(out, cost)
        return x_dev

    def step(self, x, show: bool = False):
        """One iteration (``cls_basic.py:987-1136``)."""
        if self._native:
            self._dev.run(1, graph=False)
            x_dev = self._sync_native()
            x = _like_input(x_dev, self.y)
            if show:
                self._print_step(x)
            return x
        self.u = self.Op.matvec(self.v) - self.alfa * self.u
        self.beta = _norm(self.u)
        if self.beta > 0:
            self.u = self.u / self.beta
            self.anorm = float(np.linalg.norm([self.anorm, self.alfa, self.beta, self.damp]))
            self.v = self.Op.rmatvec(self.u) - self.beta * self.v
            self.alfa = _norm(self.v)
            if self.alfa > 0:
                self.v = self.v / self.alfa
        rhobar1 = float(np.linalg.norm([self.rhobar, self.damp]))
        cs1 = self.rhobar / rhobar1
        sn1 = self.damp / rhobar1
        psi = sn1 * self.phibar
        self.phibar = cs1 * self.phibar
        rho = float(np.linalg.norm([rhobar1, self.beta]))
        cs = rhobar1 / rho
        sn = self.beta / rho
        theta = sn * self.alfa
        self.rhobar = -cs * self.alfa
        phi = cs * self.phibar
        self.phibar = sn * self.phibar
        tau = sn * phi
        t1 = phi / rho
        t2 = -theta / rho
        dknorm2 = _dot(self.w, self.w) / rho ** 2
        x = x + t1 * self.w
        self.w = self.v + t2 * self.w
        self.ddnorm = self.ddnorm + dknorm2
        if self.calc_var:
            self.var_scalar = self.var_scalar + dknorm2
        delta = self.sn2 * rho
        gambar = -self.cs2 * rho
        rhs = phi - delta * self.z
        zbar = rhs / gambar
        self.xnorm = float(np.sqrt(self.xxnorm + zbar ** 2))
        gamma = float(np.linalg.norm([gambar, theta]))
        self.cs2 = gambar / gamma
        self.sn2 = theta / gamma
        self.z = rhs / gamma
        self.xxnorm = self.xxnorm + self.z ** 2.0
        self.acond = self.anorm * np.sqrt(self.ddnorm)
        res1 = self.phibar ** 2
        self.res2 = self.res2 + psi ** 2
        self.rnorm = float(np.sqrt(res1 + self.res2))
        self.arnorm = self.alfa * abs(tau)
        r1sq = self.rnorm ** 2 - self.dampsq * self.xxnorm
        self.r1norm = float(np.sqrt(np.abs(r1sq)))
        self.cost.append(float(self.r1norm))
        if r1sq < 0:
            self.r1norm = -self.r1norm
        self.r2norm = self.rnorm
        self.test1 = self.rnorm / self.bnorm
        self.test2 = self.arnorm / self.arnorm0
        self.test3 = 1.0 / self.acond
        tt1 = self.test1 / (1.0 + self.anorm * self.xnorm / self.bnorm)
        self.rtol = self.btol + self.atol * self.anorm * self.xnorm / self.bnorm
        if self.iiter >= self.niter:
            self.istop = 7
        if 1 + self.test3 <= 1:
            self.istop = 6
        if 1 + self.test2 <= 1:
            self.istop = 5
        if 1 + tt1 <= 1:
            self.istop = 4
        if self.test3 <= self.ctol:
            self.istop = 3
        if self.test2 <= self.atol:
            self.istop = 2
        if self.test1 <= self.rtol:
            self.istop = 1
        self.iiter += 1
        if show:
            self._print_step(x)
        return x

    def run(self, x, niter: Optional[int] = None, show: bool = False, itershow=(10, 10, 10)):
        """Iterate while ``iiter < niter and istop == 0`` (``cls_basic.py:1138-1186``)."""
        niter = self.niter if niter is None else niter
        if self._native and not show and not self.callbacks and not _has_user_callback(self):
            self._dev.run(niter - self.iiter, graph=True)
            x_dev = self._sync_native()
            return _like_input(x_dev, self.y)
        while self.iiter < niter and self.istop == 0:
            x = self.step(x, show and (self.niter <= 40 or self.iiter < itershow[0]
                                       or niter - self.iiter < itershow[1] or self.iiter % itershow[2] == 0))
            self.callback(x)
        return x

    def finalize(self, show: bool = False) -> None:
        self.tend = time.time()
        self.telapsed = self.tend - self.tstart
        self.cost = np.array(self.cost)
        self.var = np.full(self.Op.shape[1], self.var_scalar) if self.calc_var else None
        if show:
            self._print_finalize()

    def solve(self, y, x0=None, damp: float = 0.0, atol: float = 1e-08, btol: float = 1e-08,
              conlim: float = 100000000.0, niter: int = 10, calc_var: bool = True, preallocate: bool = False,
              show: bool = False, itershow=(10, 10, 10)) -> Tuple:
        x = self.setup(y=y, x0=x0, damp=damp, atol=atol, btol=btol, conlim=conlim, niter=niter,
                       calc_var=calc_var, preallocate=preallocate, show=show)
        x = self.run(x, niter=niter, show=show, itershow=itershow)
        self.finalize(show)
        return (x, self.istop, self.iiter, self.r1norm, self.r2norm, self.anorm, self.acond, self.arnorm,
                self.xnorm, self.var, self.cost)
