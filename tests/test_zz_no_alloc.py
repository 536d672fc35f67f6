"""The allocation-free forward (kgb_kirchhoff_forward_static).

It is for callers that must not call cudaMalloc while they run -- a fixed
device-memory budget, memory owned by a pool or caching allocator, or a
latency-critical loop -- and keeps its scratch in a static device array of
at most 4,194,304 image points.  These tests call it through the C ABI and
hold its output to the regular forward's on two calls in a row.  Both run
the same kernels with the same scale choice, so the outputs must be equal
bit for bit (a tighter bar than the operator's 1e-5 parity tolerance).  The
larger model goes first: a scale block left over from it would then change
the second, smaller call's fixed-point scale and its result.  The file is
collected last so a failure here leaves every other test already run.
"""

import ctypes

import numpy as np
import pytest

from tests.helpers import kwargs_from_golden, load, rel

pytestmark = pytest.mark.gpu


def _operator(name):
    from pylops_gb300.waveeqprocessing import Kirchhoff

    g = load(name)
    if "trav_table" in g:  # single traveltime table of shape (ni, ns*nr)
        return Kirchhoff(g["z"], g["x"], g["t"], g["srcs"], g["recs"], float(g["vel_scalar"]), g["wav"],
                         int(g["wavc"]), mode="byot", trav=g["trav_table"], engine="cuda", dtype="float32")
    args, kw = kwargs_from_golden(g)
    return Kirchhoff(*args, engine="cuda", dtype="float32", **kw)


@pytest.mark.parametrize("name", ["k2d_kin", "k2d_dyn_ap", "k3d_dyn", "k2d_single", "k2d_single_neg"])
def test_static_forward_matches_regular_forward_twice(name):
    import torch

    from pylops_gb300 import _native

    L = _native.lib()
    K = _operator(name)
    h = K.native_handle
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    for call in range(2):  # two calls in a row, larger model first: the shared scratch must not leak state
        m = torch.as_tensor(rng.standard_normal(K.ni).astype(np.float32) * (10.0 ** (1 - call)), device="cuda")
        y_ref = torch.empty(K.shape[0], dtype=torch.float32, device="cuda")
        y_static = torch.full((K.shape[0],), float("nan"), dtype=torch.float32, device="cuda")
        _native.check(L.kgb_kirchhoff_forward(h, m.data_ptr(), y_ref.data_ptr(), stream))
        _native.check(L.kgb_kirchhoff_forward_static(h, m.data_ptr(), y_static.data_ptr(), stream))
        torch.cuda.synchronize()
        a, b = y_static.cpu().numpy(), y_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert np.array_equal(a, b), (call, rel(a, b))


def test_static_forward_rejects_operators_beyond_its_maximum():
    import torch

    from pylops_gb300 import _native

    L = _native.lib()
    h = ctypes.c_void_p()
    wav = np.ascontiguousarray(np.array([0.25, 0.5, 0.25]))
    ni = (1 << 22) + 16  # one column beyond the static maximum
    _native.check(L.kgb_kirchhoff_create(ctypes.byref(h), 1, 1, 8, ni, 16, 0.004, 0, _native.dptr(wav), 3, 1))
    try:
        t = np.zeros(ni)
        _native.check(L.kgb_kirchhoff_set_traveltimes(h, _native.dptr(t), _native.dptr(t)))
        # buffers of the full size, so that nothing could go out of bounds
        m = torch.zeros(ni, dtype=torch.float32, device="cuda")
        d = torch.zeros(8, dtype=torch.float32, device="cuda")
        rc = L.kgb_kirchhoff_forward_static(h, m.data_ptr(), d.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == _native.KGB_ERR_VALUE
        assert b"static scratch maximum" in L.kgb_last_error()
    finally:
        L.kgb_kirchhoff_destroy(h)
