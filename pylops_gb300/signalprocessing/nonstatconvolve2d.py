"""2-D non-stationary convolution (``pylops/signalprocessing/nonstatconvolve2d.py:34-300``).

``NonStationaryConvolve2D(dims, hs, ihx, ihz)`` convolves an (nx, nz) image
with filters that vary in space: ``hs`` (nhx, nhz, hx, hz) holds compact
filters (odd sizes) at the regularly sampled image points ``ihx`` x ``ihz``
and the filter at any point is their bilinear interpolation.  In image-domain
least-squares migration the filters are point-spread functions of the
Kirchhoff Hessian ``K^H K``.  Forward and adjoint run on the device
(``kgb_nsconv2d_apply``) as deterministic gathers, for every ``engine``.
"""

from __future__ import annotations

from typing import Sequence, Tuple

import numpy as np

from .. import _native
from ..linearoperator import LinearOperator
from ..utils.backend import is_torch

__all__ = ["NonStationaryConvolve2D"]


class NonStationaryConvolve2D(LinearOperator):
    def __init__(self, dims: Tuple[int, int], hs, ihx: Sequence[int], ihz: Sequence[int], engine: str = "numpy",
                 num_threads_per_blocks: Tuple[int, int] = (32, 32), dtype="float64", name: str = "C"):
        if engine not in ["numpy", "numba", "cuda"]:
            raise NotImplementedError("engine must be numpy or numba or cuda")
        hs = np.asarray(hs) if not is_torch(hs) else hs
        if hs.shape[2] % 2 == 0 or hs.shape[3] % 2 == 0:
            raise ValueError("filters hs must have odd length")
        ihx, ihz = np.asarray(ihx), np.asarray(ihz)
        if len(np.unique(np.diff(ihx))) > 1 or len(np.unique(np.diff(ihz))) > 1:
            raise ValueError("the indices of filters 'ih' must be regularly sampled")
        dims = tuple(int(d) for d in dims)
        if min(ihx) < 0 or min(ihz) < 0 or max(ihx) >= dims[0] or max(ihz) >= dims[1]:
            raise ValueError("the indices of filters 'ih' must be larger than 0 and smaller than `dims`")
        self.hs = hs
        self.hshape = tuple(hs.shape[2:])
        self.ohx, self.dhx, self.nhx = int(ihx[0]), int(ihx[1] - ihx[0]) if len(ihx) > 1 else 1, len(ihx)
        self.ohz, self.dhz, self.nhz = int(ihz[0]), int(ihz[1] - ihz[0]) if len(ihz) > 1 else 1, len(ihz)
        self.ehx, self.ehz = int(ihx[-1]), int(ihz[-1])
        self.engine = engine
        super().__init__(dtype=np.dtype(dtype), dims=dims, dimsd=dims, name=name)
        self._hs_dev = None

    def _filters(self):
        import torch

        if self._hs_dev is None:
            h = self.hs if is_torch(self.hs) else torch.from_numpy(np.ascontiguousarray(self.hs, dtype=np.float32))
            self._hs_dev = h.to(device="cuda", dtype=torch.float32).contiguous()
        return self._hs_dev

    def _apply(self, x, adjoint: bool):
        import torch

        dev = is_torch(x)
        xx = (x.to(device="cuda", dtype=torch.float32) if dev else
              torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device="cuda")).reshape(-1).contiguous()
        y = torch.empty_like(xx)
        nx, nz = self.dims
        _native.check(_native.lib().kgb_nsconv2d_apply(
            xx.data_ptr(), y.data_ptr(), self._filters().data_ptr(), nx, nz, self.nhx, self.nhz, self.hshape[0],
            self.hshape[1], float(self.ohx), float(self.ohz), float(self.dhx), float(self.dhz), int(adjoint),
            torch.cuda.current_stream().cuda_stream))
        if dev:
            return y if x.dtype == torch.float32 else y.to(x.dtype)
        return y.cpu().numpy().astype(self.dtype, copy=False)

    def _matvec(self, x):
        return self._apply(x, False)

    def _rmatvec(self, x):
        return self._apply(x, True)
