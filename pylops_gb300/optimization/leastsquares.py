"""Functional form of the preconditioned inversion
(``pylops/optimization/leastsquares.py:217-286``)."""

from typing import Optional, Tuple

from .cls_leastsquares import PreconditionedInversion

__all__ = ["preconditioned_inversion"]


def preconditioned_inversion(Op, y, P, x0: Optional = None, engine: str = "scipy", show: bool = False,
                             **kwargs_solver) -> Tuple:
    """Solve ``y = Op P p`` and return ``(P p, istop, itn, r1norm, r2norm)``."""
    psolve = PreconditionedInversion(Op)
    return psolve.solve(y, P, x0=x0, engine=engine, show=show, **kwargs_solver)
