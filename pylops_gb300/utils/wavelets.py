"""Wavelets (``pylops/utils/wavelets.py:167-205``)."""

import warnings

import numpy as np

__all__ = ["ricker"]


def _tcrop(t):
    if len(t) % 2 == 0:
        t = t[:-1]
        warnings.warn("One sample removed from time axis...")
    return t


def ricker(t, f0: float = 10, taper=None):
    """Ricker wavelet on the symmetric axis built from the positive part ``t``.

    Returns ``(w, t_symmetric, wcenter)``.
    """
    t = _tcrop(np.asarray(t))
    t = np.concatenate((np.flipud(-t[1:]), t), axis=0)
    arg = (np.pi * f0 * t) ** 2
    w = (1 - 2 * arg) * np.exp(-arg)
    wcenter = int(np.argmax(np.abs(w)))
    if taper is not None:
        w *= taper(len(t))
    return w, t, wcenter
