from . import basic, cls_basic, cls_leastsquares, leastsquares
from .basic import cgls, lsqr
from .cls_leastsquares import PreconditionedInversion
from .leastsquares import preconditioned_inversion
from .callback import Callbacks, MetricsCallback
from .cls_basic import CGLS, LSQR

__all__ = ["cgls", "lsqr", "CGLS", "LSQR", "Callbacks", "MetricsCallback", "basic", "cls_basic",
           "PreconditionedInversion", "preconditioned_inversion"]
