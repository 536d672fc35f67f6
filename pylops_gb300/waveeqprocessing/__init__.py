from .kirchhoff import Kirchhoff
from .lsm import LSM

__all__ = ["Kirchhoff", "LSM"]
