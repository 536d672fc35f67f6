from .dottest import dottest
from .tapers import taper
from .wavelets import ricker

__all__ = ["dottest", "ricker", "taper"]
