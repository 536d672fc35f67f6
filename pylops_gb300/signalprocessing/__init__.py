"""Signal-processing operators used around the Kirchhoff path."""

from .nonstatconvolve2d import NonStationaryConvolve2D

__all__ = ["NonStationaryConvolve2D"]
