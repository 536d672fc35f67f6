from .batch import KirchhoffBatch
from .kirchhoff import Kirchhoff
from .lsm import LSM

__all__ = ["Kirchhoff", "KirchhoffBatch", "LSM"]
