from . import basic, cls_basic
from .basic import cgls, lsqr
from .callback import Callbacks, MetricsCallback
from .cls_basic import CGLS, LSQR

__all__ = ["cgls", "lsqr", "CGLS", "LSQR", "Callbacks", "MetricsCallback", "basic", "cls_basic"]
