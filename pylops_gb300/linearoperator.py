"""Linear-operator algebra: the drop-in boundary of the package.

Mirrors the subset of ``pylops.LinearOperator`` (pylops/linearoperator.py)
that the Kirchhoff least-squares-migration path uses: shape/dims/dimsd,
``matvec``/``rmatvec`` with the reference's shape checks and counters
(``linearoperator.py:154-157, 489-559``), ``dot``/``@``/``*`` with
ndarray reshaping (``:612-702``), ``.H``/``.T`` (``:481``), sums, products
and scaling (``:1254-1495``).  Vectors may be numpy arrays (host) or torch
CUDA tensors (device); an operator returns the kind it was given.
"""

from __future__ import annotations

import numbers
from typing import Optional, Sequence, Tuple, Union

import numpy as np

from .utils.backend import get_array_module, is_torch

__all__ = ["LinearOperator", "aslinearoperator"]


def _tuple(d) -> Tuple[int, ...]:
    if d is None:
        return None
    if isinstance(d, numbers.Integral):
        return (int(d),)
    return tuple(int(v) for v in d)


class LinearOperator:
    """Common interface of linear operators (``pylops/linearoperator.py:54``).

    Subclasses implement ``_matvec`` and ``_rmatvec`` on flat vectors.
    """

    def __init__(
        self,
        Op=None,
        dtype=None,
        shape: Optional[Tuple[int, int]] = None,
        dims: Optional[Union[int, Sequence[int]]] = None,
        dimsd: Optional[Union[int, Sequence[int]]] = None,
        clinear: Optional[bool] = None,
        explicit: Optional[bool] = None,
        forceflat: Optional[bool] = None,
        name: Optional[str] = None,
    ) -> None:
        if Op is not None:
            dtype = Op.dtype if dtype is None else dtype
            shape = Op.shape if shape is None else shape
            dims = getattr(Op, "dims", None) if dims is None else dims
            dimsd = getattr(Op, "dimsd", None) if dimsd is None else dimsd
            self.Op = Op
        self.dtype = np.dtype(dtype if dtype is not None else np.float64)
        if dims is not None:
            self.dims = _tuple(dims)
        if dimsd is not None:
            self.dimsd = _tuple(dimsd)
        if shape is None:
            shape = (int(np.prod(self.dimsd)), int(np.prod(self.dims)))
        self.shape = (int(shape[0]), int(shape[1]))
        if dims is None:
            self.dims = (self.shape[1],)
        if dimsd is None:
            self.dimsd = (self.shape[0],)
        if int(np.prod(self.dims)) != self.shape[1] or int(np.prod(self.dimsd)) != self.shape[0]:
            raise ValueError("dims and dimsd must be consistent with shape")
        self.clinear = True if clinear is None else clinear
        self.explicit = False if explicit is None else explicit
        self.forceflat = forceflat
        self.name = name
        self.reset_count()

    # ------------------------------------------------------------ counters
    def reset_count(self) -> None:
        """Reset the matvec/rmatvec counters (``linearoperator.py:154-157``)."""
        self.matvec_count = 0
        self.rmatvec_count = 0
        self.matmat_count = 0
        self.rmatmat_count = 0

    # ------------------------------------------------------------ apply
    def _matvec(self, x):
        raise NotImplementedError

    def _rmatvec(self, x):
        raise NotImplementedError

    def matvec(self, x):
        """Forward ``y = Op x`` for a flat vector (``linearoperator.py:489-523``)."""
        M, N = self.shape
        if tuple(x.shape) != (N,) and tuple(x.shape) != (N, 1):
            raise ValueError(f"Dimension mismatch. Got {tuple(x.shape)}, but expected ({N},) or ({N}, 1).")
        y = self._matvec(x.reshape(-1))
        y = y.reshape(M) if x.ndim == 1 else y.reshape(M, 1)
        self.matvec_count += 1
        return y

    def rmatvec(self, x):
        """Adjoint ``x = Op^H y`` for a flat vector (``linearoperator.py:525-559``)."""
        M, N = self.shape
        if tuple(x.shape) != (M,) and tuple(x.shape) != (M, 1):
            raise ValueError(f"Dimension mismatch. Got {tuple(x.shape)}, but expected ({M},) or ({M}, 1).")
        y = self._rmatvec(x.reshape(-1))
        y = y.reshape(N) if x.ndim == 1 else y.reshape(N, 1)
        self.rmatvec_count += 1
        return y

    def matmat(self, X):
        """Column-by-column forward of a 2-D array (``linearoperator.py:561-585``)."""
        if X.ndim != 2 or X.shape[0] != self.shape[1]:
            raise ValueError(f"Dimension mismatch: {tuple(X.shape)} vs {self.shape}")
        ncp = get_array_module(X)
        cols = [self.matvec(X[:, j]) for j in range(X.shape[1])]
        self.matmat_count += 1
        return ncp.stack(cols, 1) if is_torch(X) else np.stack(cols, axis=1)

    def rmatmat(self, X):
        if X.ndim != 2 or X.shape[0] != self.shape[0]:
            raise ValueError(f"Dimension mismatch: {tuple(X.shape)} vs {self.shape}")
        ncp = get_array_module(X)
        cols = [self.rmatvec(X[:, j]) for j in range(X.shape[1])]
        self.rmatmat_count += 1
        return ncp.stack(cols, 1) if is_torch(X) else np.stack(cols, axis=1)

    def dot(self, x):
        """Operator product, scaling or application (``linearoperator.py:612-702``)."""
        if isinstance(x, LinearOperator):
            return _ProductLinearOperator(self, x)
        if np.isscalar(x):
            return _ScaledLinearOperator(self, x)
        if not hasattr(x, "shape"):
            x = np.asarray(x)
        if x.ndim == 1 or (x.ndim == 2 and x.shape[1] == 1 and x.shape[0] == self.shape[1]):
            return self.matvec(x)
        if tuple(x.shape) == tuple(self.dims):
            return self.matvec(x.reshape(-1)).reshape(self.dimsd)
        if x.ndim == 2:
            return self.matmat(x)
        raise ValueError(f"expected 1-d or 2-d array or matrix, got {tuple(x.shape)}")

    def __matmul__(self, x):
        if np.isscalar(x):
            raise ValueError("Scalar operands are not allowed, use '*' instead")
        return self.dot(x)

    def __rmatmul__(self, x):
        if np.isscalar(x):
            raise ValueError("Scalar operands are not allowed, use '*' instead")
        return NotImplemented

    def __mul__(self, x):
        return self.dot(x)

    def __rmul__(self, x):
        if np.isscalar(x):
            return _ScaledLinearOperator(self, x)
        return NotImplemented

    def __neg__(self):
        return _ScaledLinearOperator(self, -1)

    def __add__(self, other):
        if not isinstance(other, LinearOperator):
            return NotImplemented
        return _SumLinearOperator(self, other)

    def __sub__(self, other):
        return self.__add__(-other)

    def __pow__(self, p: int):
        if not isinstance(p, numbers.Integral) or p < 0:
            return NotImplemented
        if self.shape[0] != self.shape[1]:
            raise ValueError("square operator expected")
        return _PowerLinearOperator(self, int(p))

    # ------------------------------------------------------------ adjoint
    def _adjoint(self):
        return _AdjointLinearOperator(self)

    def adjoint(self):
        """Hermitian adjoint (``linearoperator.py:481``)."""
        return self._adjoint()

    H = property(adjoint)

    def transpose(self):
        return _TransposedLinearOperator(self)

    T = property(transpose)

    def todense(self, backend: str = "numpy"):
        """Dense matrix by applying the operator to identity columns."""
        N = self.shape[1]
        cols = []
        for j in range(N):
            e = np.zeros(N, dtype=self.dtype)
            e[j] = 1.0
            cols.append(np.asarray(self.matvec(e)))
        return np.stack(cols, axis=1)

    def __repr__(self):
        return f"<{self.shape[0]}x{self.shape[1]} {type(self).__name__} with dtype={self.dtype}>"


class _AdjointLinearOperator(LinearOperator):
    def __init__(self, A):
        super().__init__(dtype=A.dtype, shape=(A.shape[1], A.shape[0]), dims=A.dimsd, dimsd=A.dims,
                         clinear=A.clinear, name=A.name)
        self.A = A

    def _matvec(self, x):
        return self.A._rmatvec(x)

    def _rmatvec(self, x):
        return self.A._matvec(x)

    def _adjoint(self):
        return self.A


class _TransposedLinearOperator(LinearOperator):
    def __init__(self, A):
        super().__init__(dtype=A.dtype, shape=(A.shape[1], A.shape[0]), dims=A.dimsd, dimsd=A.dims,
                         clinear=A.clinear, name=A.name)
        self.A = A

    def _matvec(self, x):
        return self.A._rmatvec(x.conj()).conj()

    def _rmatvec(self, x):
        return self.A._matvec(x.conj()).conj()


class _ProductLinearOperator(LinearOperator):
    def __init__(self, A, B):
        if A.shape[1] != B.shape[0]:
            raise ValueError(f"cannot multiply {A} and {B}: shape mismatch")
        super().__init__(dtype=np.result_type(A.dtype, B.dtype), shape=(A.shape[0], B.shape[1]),
                         dims=B.dims, dimsd=A.dimsd)
        self.args = (A, B)

    def _matvec(self, x):
        return self.args[0].matvec(self.args[1].matvec(x))

    def _rmatvec(self, x):
        return self.args[1].rmatvec(self.args[0].rmatvec(x))


class _ScaledLinearOperator(LinearOperator):
    def __init__(self, A, alpha):
        super().__init__(dtype=np.result_type(A.dtype, np.asarray(alpha).dtype) if not isinstance(alpha, float)
                         else A.dtype, shape=A.shape, dims=A.dims, dimsd=A.dimsd)
        self.args = (A, alpha)

    def _matvec(self, x):
        return self.args[0].matvec(x) * self.args[1]

    def _rmatvec(self, x):
        return self.args[0].rmatvec(x) * np.conj(self.args[1])


class _SumLinearOperator(LinearOperator):
    def __init__(self, A, B):
        if A.shape != B.shape:
            raise ValueError(f"cannot add {A} and {B}: shape mismatch")
        super().__init__(dtype=np.result_type(A.dtype, B.dtype), shape=A.shape, dims=A.dims, dimsd=A.dimsd)
        self.args = (A, B)

    def _matvec(self, x):
        return self.args[0].matvec(x) + self.args[1].matvec(x)

    def _rmatvec(self, x):
        return self.args[0].rmatvec(x) + self.args[1].rmatvec(x)


class _PowerLinearOperator(LinearOperator):
    def __init__(self, A, p):
        super().__init__(dtype=A.dtype, shape=A.shape, dims=A.dims, dimsd=A.dimsd)
        self.args = (A, p)

    def _matvec(self, x):
        for _ in range(self.args[1]):
            x = self.args[0].matvec(x)
        return x

    def _rmatvec(self, x):
        for _ in range(self.args[1]):
            x = self.args[0].rmatvec(x)
        return x


class _MatrixOperator(LinearOperator):
    """Dense matrix wrapped as an operator (test helper, like ``MatrixMult``)."""

    def __init__(self, A, dtype=None):
        self.A = A
        super().__init__(dtype=dtype or A.dtype, shape=A.shape)

    def _matvec(self, x):
        A = self.A
        if is_torch(x) and not is_torch(A):
            import torch
            self.A = A = torch.as_tensor(A, device=x.device, dtype=x.dtype)
        return A @ x

    def _rmatvec(self, x):
        A = self.A
        if is_torch(x) and not is_torch(A):
            import torch
            self.A = A = torch.as_tensor(A, device=x.device, dtype=x.dtype)
        return A.conj().T @ x if not is_torch(A) else A.T.conj() @ x


def aslinearoperator(Op):
    """Wrap a dense matrix (numpy/torch) or return an operator unchanged."""
    if isinstance(Op, LinearOperator):
        return Op
    return _MatrixOperator(Op)
