"""Float64 restatement of the 2-D non-stationary convolution
(``pylops/signalprocessing/nonstatconvolve2d.py:177-272``) -- test
infrastructure: the oracle for ``kgb_nsconv2d_apply``, never the thing
measured or shipped.  Pinned to golden vectors the reference produced
(``tests/golden/nsconv2d.npz``)."""

import numpy as np


def _interp(i, o, d, n):
    # nonstatconvolve2d.py:193-215: lower index by floor, edge filter with
    # weights 1/2 outside the coarse grid
    lo = int(np.floor((i - o) / d))
    if lo < 0:
        return 0, 0, 0.5, 0.5
    if lo >= n - 1:
        return n - 1, n - 1, 0.5, 0.5
    f = (i - o) / d - lo
    return lo, lo + 1, 1.0 - f, f


def nsconv2d(x, hs, ihx, ihz, adjoint=False):
    """Forward (``adjoint=False``) or adjoint of NonStationaryConvolve2D on
    an (nx, nz) image; returns float64 (nx, nz)."""
    x = np.asarray(x, dtype=np.float64)
    nx, nz = x.shape
    hs = np.asarray(hs, dtype=np.float64)
    hx, hz = hs.shape[2:]
    ohx, dhx, nhx = ihx[0], ihx[1] - ihx[0], len(ihx)
    ohz, dhz, nhz = ihz[0], ihz[1] - ihz[0], len(ihz)
    y = np.zeros((nx, nz))
    for ix in range(nx):
        xl, xr, wl, wr = _interp(ix, ohx, dhx, nhx)
        for iz in range(nz):
            zt, zb, wt, wb = _interp(iz, ohz, dhz, nhz)
            h = wt * wl * hs[xl, zt] + wb * wl * hs[xl, zb] + wt * wr * hs[xr, zt] + wb * wr * hs[xr, zb]
            x0, x1 = max(0, ix - hx // 2), min(ix + hx // 2 + 1, nx)
            z0, z1 = max(0, iz - hz // 2), min(iz + hz // 2 + 1, nz)
            a0, a1 = max(0, -ix + hx // 2), min(hx, hx // 2 + (nx - ix))
            b0, b1 = max(0, -iz + hz // 2), min(hz, hz // 2 + (nz - iz))
            if adjoint:
                y[ix, iz] = np.sum(h[a0:a1, b0:b1] * x[x0:x1, z0:z1])
            else:
                y[x0:x1, z0:z1] += x[ix, iz] * h[a0:a1, b0:b1]
    return y
