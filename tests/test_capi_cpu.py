"""CPU-side checks of the C ABI: the library builds, loads and exports every
declared symbol; argument validation that returns before any device work;
and the host-side eikonal table builder."""

import ctypes
import os
import re

import numpy as np
import pytest

from pylops_gb300 import _native
from tests.conftest import ROOT


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(kgb_\w+)\s*\(", src, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = _native.lib()
    declared = _declared()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    # and the ctypes binding declares exactly the header's entry points
    assert set(_native.exported_symbols()) == declared


def test_version_and_error_text():
    L = _native.lib()
    assert L.kgb_version() == 100
    h = ctypes.c_void_p()
    w = np.ones(3)
    rc = L.kgb_kirchhoff_create(ctypes.byref(h), 0, 1, 10, 10, 10, 0.004, 0, _native.dptr(w), 3, 1)
    assert rc == _native.KGB_ERR_VALUE
    assert b"bad sizes" in L.kgb_last_error()
    with pytest.raises(ValueError):
        _native.check(rc)
    rc = L.kgb_kirchhoff_create(ctypes.byref(h), 1, 1, 10, 10, 10, 0.004, 0, _native.dptr(w), 3, 5)
    assert rc == _native.KGB_ERR_VALUE  # offset must be smaller than len(h)-1, like Convolve1D
    rc = L.kgb_kirchhoff_create(ctypes.byref(h), 1, 1, 10, 10, 3, 0.004, 0, _native.dptr(w), 3, 1)
    assert rc == _native.KGB_ERR_VALUE  # ni not a multiple of nz
    assert L.kgb_kirchhoff_forward(None, None, None, None) == _native.KGB_ERR_STATE
    assert L.kgb_solver_create(None, None, 0) == _native.KGB_ERR_VALUE


def test_eikonal_matches_analytic_constant_velocity():
    """Same check as the reference's test_traveltime_table (decimal=2),
    which is vacuous there without scikit-fmm."""
    from pylops_gb300.waveeqprocessing.kirchhoff import Kirchhoff

    z = np.arange(20) * 2.0
    x = np.arange(12) * 1.0
    s = np.vstack((np.linspace(0, 11, 6), 2 * np.ones(6)))
    r = np.vstack((np.linspace(0, 11, 2), 2 * np.ones(2)))
    te_s, te_r, de_s, _, _, _ = Kirchhoff._traveltime_table(z, x, s, r, 500 * np.ones((12, 20)), mode="eikonal")
    ta_s, ta_r, da_s, _, _, _ = Kirchhoff._traveltime_table(z, x, s, r, 500.0, mode="analytic")
    np.testing.assert_array_almost_equal(ta_s, te_s, decimal=2)
    np.testing.assert_array_almost_equal(ta_r, te_r, decimal=2)
    # on-grid source in a large homogeneous grid: the level set starts half a
    # cell from the source node (scikit-fmm's convention), so arrival times are
    # early by up to about one cell time; the marching error stays below that
    z = np.arange(101) * 5.0
    x = np.arange(121) * 5.0
    src = np.array([[300.0], [0.0]])
    te, _, de, _, _, _ = Kirchhoff._traveltime_table(z, x, src, src, 2000.0 * np.ones((121, 101)), mode="eikonal")
    ta, _, da, _, _, _ = Kirchhoff._traveltime_table(z, x, src, src, 2000.0, mode="analytic")
    far = da[:, 0] > 100.0
    cell_time = 5.0 / 2000.0
    assert np.max(np.abs(te[far, 0] - ta[far, 0])) < cell_time
    assert np.max(np.abs(de[far, 0] - da[far, 0])) < 5.0


def test_eikonal_rejects_bad_input():
    L = _native.lib()
    dims = np.array([4, 4], dtype=np.int32)
    h = np.array([1.0, 1.0])
    v = np.ones(16)
    pts = np.array([5, 0], dtype=np.int32)
    out = np.zeros(16)
    rc = L.kgb_eikonal_tables(2, _native.iptr(dims), _native.dptr(h), _native.dptr(v), 1, _native.iptr(pts),
                              _native.dptr(out), None, 2, 1)
    assert rc == _native.KGB_ERR_VALUE
    v[3] = -1.0
    pts = np.array([1, 1], dtype=np.int32)
    rc = L.kgb_eikonal_tables(2, _native.iptr(dims), _native.dptr(h), _native.dptr(v), 1, _native.iptr(pts),
                              _native.dptr(out), None, 2, 1)
    assert rc == _native.KGB_ERR_VALUE
