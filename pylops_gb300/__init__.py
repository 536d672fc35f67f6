"""GB300-native Kirchhoff demigration/migration and least-squares migration.

A drop-in for the PyLops path ``pylops.waveeqprocessing.Kirchhoff`` ->
``pylops.optimization`` (CGLS/LSQR) -> ``pylops.waveeqprocessing.LSM``:
same constructors, ``LinearOperator`` behaviour and solver API, computed by
hand-written sm_103a CUDA kernels in ``libpylops_gb300.so``.
"""

from .linearoperator import LinearOperator, aslinearoperator
from . import utils
from . import waveeqprocessing
from . import optimization
from . import basicoperators
from .torchoperator import TorchOperator

__version__ = "0.1.0"

__all__ = ["LinearOperator", "aslinearoperator", "utils", "waveeqprocessing", "optimization", "basicoperators",
           "TorchOperator"]
