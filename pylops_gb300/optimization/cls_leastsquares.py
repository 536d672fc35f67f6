"""Preconditioned inversion (``pylops/optimization/cls_leastsquares.py:768-1021``).

Solves ``y = Op P p`` and returns ``x = P p``.  ``engine='scipy'`` with
numpy data runs ``scipy.sparse.linalg.lsqr`` on ``Op @ P`` (which applies
the operator through ``matvec``/``rmatvec``); ``engine='pylops'`` or torch
data runs this package's ``cgls``, which keeps the whole solve on the
device when ``Op`` is a :class:`~pylops_gb300.waveeqprocessing.Kirchhoff`
and ``P`` a real :class:`~pylops_gb300.basicoperators.Diagonal` (the
right preconditioner of the captured solver iteration).
"""

from __future__ import annotations

import time
from typing import Optional, Tuple

import numpy as np

from ..utils.backend import get_array_module
from .basesolver import Solver, _units

__all__ = ["PreconditionedInversion"]


class PreconditionedInversion(Solver):
    def _print_setup(self) -> None:
        self._print_solver(nbar=65)
        print(f"Prec={self.P}")
        print("-" * 65)

    def _print_finalize(self) -> None:
        print(f"\nTotal time (s) = {self.telapsed:.2f}")
        print("-" * 65 + "\n")

    def memory_usage(self, show: bool = False, unit: str = "B") -> float:
        nbytes = np.dtype(self.Op.dtype).itemsize
        memuse = self.Op.shape[0] * nbytes
        memuse += (2 * self.Op.shape[1] + 3 * self.Op.shape[0]) * nbytes
        memuse += (3 * self.Op.shape[1]) * nbytes
        if show:
            print(f"{type(self).__name__} will use {memuse / _units[unit]:.2f} {unit} of memory")
        return memuse

    def setup(self, y, P, show: bool = False) -> None:
        self.y = y
        self.P = P
        self.ncp = get_array_module(y)
        self.POp = self.Op @ P
        if show:
            self._print_setup()

    def step(self) -> None:
        raise NotImplementedError("PreconditionedInversion uses as default the scipy.sparse.linalg.lsqr solver, "
                                  "therefore the step method is not implemented. Use directly run or solve.")

    def run(self, x, engine: str = "scipy", show: bool = False, **kwargs_solver) -> Tuple:
        if engine == "scipy" and self.ncp == np:
            from scipy.sparse.linalg import lsqr as sp_lsqr

            if show:
                kwargs_solver["show"] = 1
            pinv, istop, itn, r1norm, r2norm = sp_lsqr(self.POp, self.y, x0=x, **kwargs_solver)[0:5]
        elif engine == "pylops" or self.ncp != np:
            from .basic import cgls

            if show:
                kwargs_solver["show"] = True
            pinv, istop, itn, r1norm, r2norm = cgls(self.POp, self.y, x0=x, **kwargs_solver)[0:5]
        else:
            raise NotImplementedError("Engine must be scipy or pylops")
        xinv = self.P.matvec(pinv)
        return xinv, istop, itn, r1norm, r2norm

    def finalize(self, show: bool = False) -> None:
        self.tend = time.time()
        self.telapsed = self.tend - self.tstart
        if show:
            self._print_finalize()

    def solve(self, y, P, x0: Optional = None, engine: str = "scipy", show: bool = False,
              **kwargs_solver) -> Tuple:
        """Returns ``(xinv, istop, itn, r1norm, r2norm)``."""
        self.setup(y=y, P=P, show=show)
        x, istop, itn, r1norm, r2norm = self.run(x0, engine=engine, show=show, **kwargs_solver)
        self.finalize(show)
        return x, istop, itn, r1norm, r2norm
