"""Least-squares migration wrapper (``pylops/waveeqprocessing/lsm.py:13-174``)."""

from typing import Callable, Optional

from scipy.sparse.linalg import lsqr

from ..utils import dottest as Dottest
from .kirchhoff import Kirchhoff

__all__ = ["LSM"]


class LSM:
    """Kirchhoff least-squares migration.

    ``LSM(z, x, t, srcs, recs, vel, wav, wavcenter, y=None, kind='kirchhoff',
    dottest=False, **kwargs_mod)`` builds ``self.Demop`` (a GB300
    :class:`Kirchhoff`); ``solve(d, solver=scipy.sparse.linalg.lsqr, **kw)``
    inverts it.  The default solver is scipy's, as in the reference
    (``lsm.py:147-174``); pass :func:`pylops_gb300.optimization.lsqr` for the
    device-resident solver.
    """

    def __init__(self, z, x, t, srcs, recs, vel, wav, wavcenter: int, y=None, kind: str = "kirchhoff",
                 dottest: bool = False, **kwargs_mod) -> None:
        self.y, self.x, self.z = y, x, z
        if kind == "kirchhoff":
            self.Demop = Kirchhoff(z, x, t, srcs, recs, vel, wav, wavcenter, y=y, **kwargs_mod)
        else:
            raise NotImplementedError("kind must be kirchhoff or twowayac")
        if dottest:
            # the operator computes in float32, so the adjointness check uses a
            # float32 tolerance (the reference's 1e-6 default assumes float64)
            Dottest(self.Demop, self.Demop.shape[0], self.Demop.shape[1], rtol=1e-4, raiseerror=True, verb=True)

    def solve(self, d, solver: Callable = lsqr, **kwargs_solver):
        minv = solver(self.Demop, d.ravel(), **kwargs_solver)[0]
        if self.y is None:
            return minv.reshape(len(self.x), len(self.z))
        return minv.reshape(len(self.y), len(self.x), len(self.z))
