"""1-D tapers (``pylops/utils/tapers.py:18-150``); the Kirchhoff aperture
taper is ``taper(41, 20, 'hanning')[20:]`` (``kirchhoff.py:412``)."""

import numpy as np

__all__ = ["hanningtaper", "cosinetaper", "taper"]


def hanningtaper(nmask: int, ntap: int):
    if ntap > 0 and (nmask // ntap) < 2:
        ntap_min = nmask // 2 if nmask % 2 == 0 else (nmask - 1) // 2
        raise ValueError(f"ntap={ntap} must be smaller or equal than {ntap_min}")
    han = np.hanning(ntap * 2 - 1)
    st = han[:ntap]
    return np.concatenate([st, np.ones(nmask - 2 * ntap), np.flipud(st)])


def cosinetaper(nmask: int, ntap: int, square: bool = False, exponent=None):
    ntap = 0 if ntap == 1 else ntap
    if exponent is None:
        exponent = 1 if not square else 2
    n = ntap * 2 - 1
    win = (0.5 * (np.cos((np.arange(n) - (ntap * 2 - 2) / 2) * np.pi / ((ntap * 2 - 2) / 2)) + 1.0)) ** exponent
    st = win[:ntap]
    return np.concatenate([st, np.ones(nmask - 2 * ntap), np.flipud(st)])


def taper(nmask: int, ntap: int, tapertype: str):
    if tapertype == "hanning":
        return hanningtaper(nmask, ntap)
    if tapertype == "cosine":
        return cosinetaper(nmask, ntap, False)
    if tapertype == "cosinesquare":
        return cosinetaper(nmask, ntap, True)
    if tapertype == "cosinesqrt":
        return cosinetaper(nmask, ntap, False, 0.5)
    return np.ones(nmask)
