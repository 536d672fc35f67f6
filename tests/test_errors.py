"""Error behaviour of the drop-in, as the reference raises it
(kirchhoff.py:303-362, 1003-1046; linearoperator.py matvec/rmatvec shape
checks).  The constructor's checks run before any device work, so the first
tests need no GPU; the others reach the library's argument checks."""

import numpy as np
import pytest

from tests.helpers import kwargs_from_golden, load


def _args():
    return kwargs_from_golden(load("k2d_kin"))


def test_unknown_engine_raises_keyerror():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = _args()
    with pytest.raises(KeyError):
        Kirchhoff(*args, engine="fortran", **kw)


def test_unknown_mode_raises_notimplemented():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = _args()
    kw["mode"] = "raytrace"
    with pytest.raises(NotImplementedError):
        Kirchhoff(*args, **kw)


def test_dynamic_single_table_raises_notimplemented():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    g = load("k2d_single")
    with pytest.raises(NotImplementedError):
        Kirchhoff(g["z"], g["x"], g["t"], g["srcs"], g["recs"], 500.0, g["wav"], int(g["wavc"]), mode="byot",
                  trav=g["trav_table"], dynamic=True, amp=g["trav_table"])


@pytest.mark.gpu
def test_wrong_vector_sizes_raise_valueerror():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = _args()
    K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    with pytest.raises(ValueError):
        K.matvec(np.zeros(K.shape[1] + 1, dtype=np.float32))
    with pytest.raises(ValueError):
        K.rmatvec(np.zeros(K.shape[0] - 1, dtype=np.float32))


@pytest.mark.gpu
def test_non_finite_traveltimes_raise_valueerror():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = _args()
    K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    ts = np.array(K.trav_srcs, copy=True)
    ts[3, 0] = np.nan
    K.trav_srcs = ts
    with pytest.raises(ValueError, match="non-finite"):
        K @ np.ones(K.shape[1], dtype=np.float32)


@pytest.mark.gpu
def test_library_rejects_bad_arguments_with_messages():
    import ctypes

    from pylops_gb300 import _native

    L = _native.lib()
    h = ctypes.c_void_p()
    wav = np.ones(3)
    # ns = 0
    rc = L.kgb_kirchhoff_create(ctypes.byref(h), 0, 4, 50, 100, 10, 0.004, 0, _native.dptr(wav), 3, 1)
    assert rc != 0 and L.kgb_last_error()
    # odd filter check of the non-stationary convolution
    rc = L.kgb_nsconv2d_apply(None, None, None, 8, 8, 2, 2, 4, 5, 0.0, 0.0, 4.0, 4.0, 0, None)
    assert rc != 0
    with pytest.raises(ValueError):
        _native.check(rc)
