"""Diagonal operator (``pylops/basicoperators/diagonal.py:14-105``).

``Diagonal(d)`` applies ``y = d * x`` (adjoint ``conj(d) * x``).  With
``dims`` and ``axis`` the diagonal is broadcast along one axis of a model of
shape ``dims``.  Numpy or torch inputs; a numpy diagonal is copied to the
device of a torch input on first use.  As the right preconditioner of a
Kirchhoff operator (``Kop * Diagonal(p)``) the CGLS/LSQR device path folds it
into the captured solver iteration.
"""

from __future__ import annotations

from typing import Optional, Sequence, Union

import numpy as np

from ..linearoperator import LinearOperator
from ..utils.backend import is_torch

__all__ = ["Diagonal"]


class Diagonal(LinearOperator):
    def __init__(self, diag, dims: Optional[Union[int, Sequence[int]]] = None, axis: int = -1,
                 dtype="float64", name: str = "D"):
        self.diag = diag
        self.axis = axis
        if dims is None:
            dims = tuple(diag.shape)
            self._bshape = None
        else:
            dims = (int(dims),) if np.isscalar(dims) else tuple(int(d) for d in dims)
            b = [1] * len(dims)
            b[axis] = dims[axis]
            self._bshape = tuple(b)
        self._dev = None
        n = int(np.prod(dims))
        super().__init__(dtype=np.dtype(dtype), shape=(n, n), dims=dims, dimsd=dims, name=name)
        self.complex = bool(np.iscomplexobj(diag)) if not is_torch(diag) else bool(diag.is_complex())

    def _d(self, x):
        d = self.diag
        if is_torch(x) and not is_torch(d):
            import torch

            if self._dev is None or self._dev.device != x.device:
                dd = np.asarray(d)
                self._dev = torch.as_tensor(dd if np.iscomplexobj(dd) else dd.astype(np.float32)
                                            if x.dtype == torch.float32 else dd, device=x.device)
            d = self._dev
        elif not is_torch(x) and is_torch(d):
            d = d.cpu().numpy()
        return d

    def _apply(self, x, conj: bool):
        d = self._d(x)
        if conj and self.complex:
            d = d.conj()
        if self._bshape is None:
            return d.reshape(-1) * x.reshape(-1)
        y = d.reshape(self._bshape) * x.reshape(self.dims)
        return y.reshape(-1)

    def _matvec(self, x):
        return self._apply(x, False)

    def _rmatvec(self, x):
        return self._apply(x, True)

    def matrix(self):
        """Dense diagonal as a numpy array."""
        d = self.diag.cpu().numpy() if is_torch(self.diag) else np.asarray(self.diag)
        if self._bshape is not None:
            d = np.broadcast_to(d.reshape(self._bshape), self.dims)
        return np.diag(d.reshape(-1))
