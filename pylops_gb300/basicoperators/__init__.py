"""Basic operators used around the Kirchhoff path."""

from .diagonal import Diagonal

__all__ = ["Diagonal"]
