"""Adjointness test (``pylops/utils/dottest.py:10-132``)."""

from typing import Optional

import numpy as np

from .backend import is_torch, to_numpy

__all__ = ["dottest"]


def dottest(Op, nr: Optional[int] = None, nc: Optional[int] = None, rtol: float = 1e-6,
            atol: float = 1e-21, complexflag: int = 0, raiseerror: bool = True, verb: bool = False,
            backend: str = "numpy", seed: Optional[int] = None) -> bool:
    """Check ``(Op u)^H v == u^H (Op^H v)`` with random ``u``, ``v``.

    ``backend='torch'`` draws the vectors on the CUDA device.  The two inner
    products are taken in float64.
    """
    if nr is None:
        nr = Op.shape[0]
    if nc is None:
        nc = Op.shape[1]
    if (nr, nc) != Op.shape:
        raise AssertionError("Provided nr and nc do not match operator shape")
    if complexflag != 0:
        raise NotImplementedError("only real operators are supported")
    rng = np.random.default_rng(seed)
    rdtype = np.ones(1, Op.dtype).real.dtype
    u = rng.standard_normal(nc).astype(rdtype)
    v = rng.standard_normal(nr).astype(rdtype)
    if backend in ("torch", "cuda"):
        import torch

        u = torch.as_tensor(u, device="cuda")
        v = torch.as_tensor(v, device="cuda")
    y = Op.matvec(u)
    x = Op.rmatvec(v)
    yy = float(np.dot(to_numpy(y).astype(np.float64), to_numpy(v).astype(np.float64)))
    xx = float(np.dot(to_numpy(u).astype(np.float64), to_numpy(x).astype(np.float64)))
    passed = bool(np.isclose(xx, yy, rtol, atol))
    if (not passed and raiseerror) or verb:
        status = "passed" if passed else "failed"
        msg = f"Dot test {status}, v^H(Opu)={yy} - u^H(Op^Hv)={xx}"
        if not passed and raiseerror:
            raise AssertionError(msg)
        print(msg)
    return passed
