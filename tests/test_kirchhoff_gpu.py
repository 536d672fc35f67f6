"""Parity of the CUDA Kirchhoff operator with the reference (golden vectors)
and with the FP64 oracle, plus dot tests, determinism and the device path.

Tolerance: 1e-5 relative L2 in float32 against float64 results, the bar the
reference-parity requirement states; the spreading/gathering kernels alone
are held to the same bound.
"""

import numpy as np
import pytest

from oracle import kirchhoff_oracle as ko
from tests.helpers import GOLDEN_CASES, kwargs_from_golden, load, rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _op(g, dtype="float32"):
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = kwargs_from_golden(g)
    return Kirchhoff(*args, engine="cuda", dtype=dtype, **kw)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_forward_adjoint_match_reference(name):
    g = load(name)
    K = _op(g)
    assert K.shape == (g["fwd"].size, g["adj"].size)
    y = K @ g["m_in"].astype(np.float32)
    x = K.H @ g["d_in"].astype(np.float32)
    assert rel(y, g["fwd"]) < TOL, rel(y, g["fwd"])
    assert rel(x, g["adj"]) < TOL, rel(x, g["adj"])


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_forward_variants_match_reference(name, variant):
    """Every forward kernel variant against the reference, bitwise repeatable."""
    g = load(name)
    K = _op(g)
    K.set_spread_variant(variant)
    y = K @ g["m_in"].astype(np.float32)
    assert rel(y, g["fwd"]) < TOL, rel(y, g["fwd"])
    assert rel(K.spread(g["m_in"]), g["spread"]) < TOL
    assert np.array_equal(y, K @ g["m_in"].astype(np.float32))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_spread_gather_match_reference(name):
    g = load(name)
    K = _op(g)
    assert rel(K.spread(g["m_in"]), g["spread"]) < TOL
    assert rel(K.gather(g["d_in"]), g["gather"]) < TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_dottest(name):
    from pylops_gb300.utils import dottest

    K = _op(load(name))
    assert dottest(K, rtol=1e-5, seed=3)
    assert dottest(K, rtol=1e-5, seed=4, backend="torch")


def _grid_100x200(nz=100, nx=200, ns=10, nr=50, nt=651, dynamic=False, angleaperture=90.0, aperture=None):
    z = np.arange(nz) * 4.0
    x = np.arange(nx) * 4.0
    t = np.arange(nt) * 0.004
    srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
    recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
    wav, _, wc = ko.ricker(t[:41], f0=20)
    rng = np.random.default_rng(0)
    refl = np.zeros((nx, nz))
    for iz in (25, 50, 75):
        refl[:, iz] = rng.standard_normal()
    for ix in range(nx):  # 10 degree dipping reflector
        iz = int(10 + ix * np.tan(np.deg2rad(10.0)))
        if iz < nz:
            refl[ix, iz] += rng.standard_normal()
    return dict(z=z, x=x, t=t, srcs=srcs, recs=recs, wav=wav, wc=wc, vel=2000.0, dynamic=dynamic,
                angleaperture=angleaperture, aperture=aperture, m=refl.ravel(),
                d=rng.standard_normal(ns * nr * nt))


@pytest.mark.parametrize("dynamic,angleaperture,aperture", [(False, 90.0, None), (True, 30.0, None),
                                                            (True, None, 1.5)])
def test_100x200_grid_against_oracle(dynamic, angleaperture, aperture):
    """100x200 grid at 4 m, 10x50 traces, nt=651, against the oracle."""
    from pylops_gb300.waveeqprocessing import Kirchhoff

    c = _grid_100x200(dynamic=dynamic, angleaperture=angleaperture, aperture=aperture)
    args = (c["z"], c["x"], c["t"], c["srcs"], c["recs"], c["vel"], c["wav"], c["wc"])
    kw = dict(mode="analytic", dynamic=dynamic, angleaperture=angleaperture, aperture=aperture)
    K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    O = ko.KirchhoffOracle(*args, **kw)
    x = K.H @ c["d"].astype(np.float32)
    assert rel(x, O.rmatvec(c["d"])) < TOL
    yo = O.matvec(c["m"])
    mr = np.random.default_rng(5).standard_normal(K.ni)  # dense model as well
    yr = O.matvec(mr)
    for variant in (0, 1, 2):
        K.set_spread_variant(variant)
        y = K @ c["m"].astype(np.float32)
        assert rel(y, yo) < TOL, (variant, rel(y, yo))
        y = K @ mr.astype(np.float32)
        assert rel(y, yr) < TOL, (variant, rel(y, yr))


@pytest.mark.parametrize("sign", [1.0, -1.0, 0.0])
def test_fixed_point_carries_against_oracle(sign):
    """The forward accumulates 30-bit contributions into 64-bit bins whose
    low 32-bit words start at 2^31; a constant-sign model makes every bin
    collect many same-sign contributions close to the scale bound, so the
    low words wrap and the carry/borrow into the high words runs (sign 0: a
    mixed-sign model with one dominant point, mostly small contributions).
    Against the float64 oracle, both forward variants."""
    from pylops_gb300.waveeqprocessing import Kirchhoff

    for dynamic in (False, True):
        c = _grid_100x200(dynamic=dynamic, angleaperture=None if not dynamic else 60.0)
        args = (c["z"], c["x"], c["t"], c["srcs"], c["recs"], c["vel"], c["wav"], c["wc"])
        kw = dict(mode="analytic", dynamic=dynamic, angleaperture=90.0 if not dynamic else 60.0)
        K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
        O = ko.KirchhoffOracle(*args, **kw)
        if sign:
            m = np.full(K.ni, sign)
        else:
            m = np.random.default_rng(8).standard_normal(K.ni) * 1e-3
            m[K.ni // 2] = 50.0
        # the spreading alone: the zero-mean wavelet would cancel most of a
        # constant-sign trace and measure float32 conditioning, not the sums
        yo = O.spread(m)
        for variant in (0, 1):
            K.set_spread_variant(variant)
            y = K.spread(m.astype(np.float32))
            assert rel(y, yo) < TOL, (dynamic, variant, rel(y, yo))


def test_negative_two_table_times_against_oracle():
    """Source and receiver tables whose sums reach below zero (user tables)
    take the general index path: -dt < ts + tr < 0 gives the reference's
    index 0 with a negative interpolation weight, so a contribution can be
    twice the model value times the weight.  Forward (both variants,
    including a model with one dominant point), spreading and adjoint
    against the float64 oracle on the same shifted tables."""
    g = load("k2d_kin")
    K = _op(g)
    O = ko.KirchhoffOracle(g["z"], g["x"], g["t"], g["srcs"], g["recs"], float(g["vel_scalar"]), g["wav"],
                           int(g["wavc"]))
    dt = float(g["t"][1] - g["t"][0])
    ts = np.asarray(K.trav_srcs, dtype=np.float64)
    tr = np.asarray(K.trav_recs, dtype=np.float64)
    shift = ts.min() + tr.min() + 0.5 * dt  # smallest sum becomes -dt/2
    K.trav_srcs = ts - shift
    O.trav_srcs = np.asarray(O.trav_srcs) - shift
    assert K.info()["nonneg"] == 0
    rng = np.random.default_rng(12)
    m = rng.standard_normal(K.ni)
    m_spiky = 1e-3 * rng.standard_normal(K.ni)
    m_spiky[K.ni // 3] = 40.0
    d = rng.standard_normal(K.shape[0])
    for variant in (0, 1):
        K.set_spread_variant(variant)
        for mm in (m, m_spiky):
            assert rel(K @ mm.astype(np.float32), O.matvec(mm)) < TOL, variant
            assert rel(K.spread(mm.astype(np.float32)), O.spread(mm)) < TOL, variant
    assert rel(K.H @ d.astype(np.float32), O.rmatvec(d)) < TOL


def test_bitwise_determinism():
    c = _grid_100x200(dynamic=True, angleaperture=40.0)
    from pylops_gb300.waveeqprocessing import Kirchhoff

    K = Kirchhoff(c["z"], c["x"], c["t"], c["srcs"], c["recs"], c["vel"], c["wav"], c["wc"], mode="analytic",
                  dynamic=True, angleaperture=40.0, dtype="float32")
    m = c["m"].astype(np.float32)
    d = c["d"].astype(np.float32)
    for variant in (0, 1, 2):
        K.set_spread_variant(variant)
        ys = [K @ m for _ in range(3)]
        for y in ys[1:]:
            assert np.array_equal(y, ys[0])
    xs = [K.H @ d for _ in range(3)]
    for x in xs[1:]:
        assert np.array_equal(x, xs[0])


def test_torch_device_path_matches_host_path():
    import torch

    g = load("k2d_dyn_ap")
    K = _op(g)
    m = g["m_in"].astype(np.float32)
    d = g["d_in"].astype(np.float32)
    yh = K @ m
    xh = K.H @ d
    yd = K @ torch.as_tensor(m, device="cuda")
    xd = K.H @ torch.as_tensor(d, device="cuda")
    assert yd.is_cuda and xd.is_cuda
    assert np.array_equal(yd.cpu().numpy(), yh)
    assert np.array_equal(xd.cpu().numpy(), xh)


@pytest.mark.parametrize("dynamic,variant", [(True, 0), (False, 0), (True, 1)])
def test_chunked_host_path_matches_device_path(dynamic, variant):
    """The host-buffer calls run the forward in receiver-group chunks on two
    streams and the adjoint's correlation in source chunks, overlapped with
    the copies; 37 receivers make a ragged last group and more groups than
    chunks.  Variant 1 takes the unchunked host path.  Bitwise equal to the
    device calls."""
    import torch

    from pylops_gb300.utils.wavelets import ricker
    from pylops_gb300.waveeqprocessing import Kirchhoff

    z, x = np.arange(60) * 5.0, np.arange(90) * 5.0
    t = np.arange(400) * 0.002
    wav, _, wc = ricker(t[:31], f0=20)
    srcs = np.vstack((np.linspace(0, x[-1], 5), np.zeros(5)))
    recs = np.vstack((np.linspace(0, x[-1], 37), np.zeros(37)))
    vel = 1500.0 + 2.0 * np.broadcast_to(z[None, :], (90, 60))
    K = Kirchhoff(z, x, t, srcs, recs, np.ascontiguousarray(vel), wav, wc, mode="eikonal", dynamic=dynamic,
                  engine="cuda", dtype="float32")
    K.set_spread_variant(variant)
    rng = np.random.default_rng(4)
    m = rng.standard_normal(K.ni).astype(np.float32)
    d = rng.standard_normal(K.shape[0]).astype(np.float32)
    for _ in range(2):  # the second call reuses streams, events and pinned blocks
        yh, xh = K @ m, K.H @ d
        yd = (K @ torch.as_tensor(m, device="cuda")).cpu().numpy()
        xd = (K.H @ torch.as_tensor(d, device="cuda")).cpu().numpy()
        assert np.array_equal(yh, yd)
        assert np.array_equal(xh, xd)


def test_table_reassignment_refreshes_device_copy():
    """The reference's tests reassign trav_srcs/trav_recs after construction."""
    g = load("k2d_kin")
    K = _op(g)
    y0 = K @ g["m_in"]
    K.trav_srcs = np.asarray(K.trav_srcs) * 1.1
    y1 = K @ g["m_in"]
    O = ko.KirchhoffOracle(g["z"], g["x"], g["t"], g["srcs"], g["recs"], float(g["vel_scalar"]), g["wav"],
                           int(g["wavc"]))
    O.trav_srcs = O.trav_srcs * 1.1
    assert rel(y1, O.matvec(g["m_in"])) < TOL
    assert rel(y0, y1) > 1e-2


def test_wavelet_operator_matches_reference_convolve1d():
    """Kirchhoff.cop against the reference's Convolve1D golden vectors."""
    import torch

    from pylops_gb300 import _native
    from pylops_gb300.waveeqprocessing import Kirchhoff
    import ctypes

    g = load("convolve1d")
    for key in sorted(k[2:] for k in g if k.startswith("h_")):
        nh, off = map(int, key.split("_"))
        h, xin = g["h_" + key], g["x_" + key]
        hnd = ctypes.c_void_p()
        hh = np.ascontiguousarray(h, dtype=np.float64)
        L = _native.lib()
        _native.check(L.kgb_kirchhoff_create(ctypes.byref(hnd), 5, 1, xin.shape[1], 4, 2, 0.004, 0,
                                             _native.dptr(hh), nh, off))
        try:
            xd = torch.as_tensor(xin.astype(np.float32), device="cuda").contiguous()
            for adj, ref in ((0, g["fwd_" + key]), (1, g["adj_" + key])):
                yd = torch.empty_like(xd)
                _native.check(L.kgb_kirchhoff_wavelet(hnd, xd.data_ptr(), yd.data_ptr(), adj, 0))
                torch.cuda.synchronize()
                assert rel(yd.cpu().numpy(), ref) < 1e-6, (key, adj)
        finally:
            L.kgb_kirchhoff_destroy(hnd)
    del Kirchhoff


def test_eikonal_operator_builds_and_passes_dottest():
    from pylops_gb300.utils import dottest
    from pylops_gb300.waveeqprocessing import Kirchhoff

    nz, nx = 40, 60
    z = np.arange(nz) * 5.0
    x = np.arange(nx) * 5.0
    t = np.arange(300) * 0.002
    vel = 1500.0 + 0.5 * z[None, :] * np.ones((nx, 1))
    srcs = np.vstack((np.linspace(x[0], x[-1], 4), np.zeros(4)))
    recs = np.vstack((np.linspace(x[0], x[-1], 16), np.zeros(16)))
    wav, _, wc = ko.ricker(t[:41], f0=15)
    K = Kirchhoff(z, x, t, srcs, recs, vel, wav, wc, mode="eikonal", dynamic=True, angleaperture=60.0,
                  dtype="float32")
    assert dottest(K, rtol=1e-5, seed=0)
    # and against the oracle fed the identical tables through byot
    O = ko.KirchhoffOracle(z, x, t, srcs, recs, vel, wav, wc, mode="byot", dynamic=True,
                           trav=(K.trav_srcs, K.trav_recs), amp=(K.amp_srcs, K.amp_recs),
                           angleaperture=60.0)
    # eikonal mode computes gradients with spacing; byot without: feed angles directly
    O.angle_srcs, O.angle_recs = K.angle_srcs, K.angle_recs
    m = np.random.default_rng(1).standard_normal(K.ni)
    assert rel(K @ m.astype(np.float32), O.matvec(m)) < TOL


def test_empty_model_and_out_of_range_times():
    """All-zero model gives zero data; traveltimes beyond the record give no
    contribution (valid range 0 <= it < nt-1, kirchhoff.py:746)."""
    g = load("k2d_kin")
    K = _op(g)
    assert np.all(K @ np.zeros(K.ni, np.float32) == 0)
    K.trav_srcs = np.asarray(K.trav_srcs) + 10.0  # every time far past nt*dt
    assert np.all(K @ g["m_in"].astype(np.float32) == 0)
    assert np.all(K.H @ g["d_in"].astype(np.float32) == 0)


@pytest.mark.parametrize("dynamic", [False, True])
def test_split_accumulation_equals_carry_accumulation_bitwise(dynamic):
    """The forward's split accumulation (two fire-and-forget 32-bit atomics
    per contribution, wide contributions in a 64-bit global accumulator) sums
    the same rounded contributions exactly, so its traces equal the carry
    accumulation's (variant 3) bit for bit: a dense model, a model with one
    dominant point (wide contributions), and again after them (the global
    accumulator must be left zero)."""
    import torch

    from pylops_gb300.waveeqprocessing import Kirchhoff

    # 40 x 64 traces: enough (source, group of 8 receivers) blocks to fill the
    # GPU, so the forward runs groups of 8, the shape the split kernels serve
    c = _grid_100x200(ns=40, nr=64, dynamic=dynamic, angleaperture=None if not dynamic else 60.0)
    args = (c["z"], c["x"], c["t"], c["srcs"], c["recs"], c["vel"], c["wav"], c["wc"])
    kw = dict(mode="analytic", dynamic=dynamic, angleaperture=90.0 if not dynamic else 60.0)
    K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    info = K.info()
    assert info["spread_split"] == 1 and 0 < info["max_bin_count"] <= 65535, info
    rng = np.random.default_rng(12)
    dense = rng.standard_normal(K.ni).astype(np.float32)
    spiky = (rng.standard_normal(K.ni) * 1e-3).astype(np.float32)
    spiky[K.ni // 2 + 37] = 50.0
    for m in (dense, spiky, dense):
        mt = torch.as_tensor(m, device="cuda")
        K.set_spread_variant(0)
        a = (K @ mt).cpu().numpy()
        K.set_spread_variant(3)
        b = (K @ mt).cpu().numpy()
        assert np.array_equal(a, b)
    K.set_spread_variant(0)
    O = ko.KirchhoffOracle(*args, **kw)
    assert rel(K @ spiky, O.matvec(spiky.astype(np.float64))) < TOL


@pytest.mark.parametrize("case", ["k2d_dyn_ap", "k2d_dyn_noap", "k3d_dyn", "k2d_dyn_byot", "grid_60", "grid_ap"])
@pytest.mark.parametrize("bf16", [False, True])
def test_adjoint_variants_equal_bitwise(case, bf16):
    """The three adjoint kernels -- records loaded in the gather (0), the next
    active source's record in flight (1), records staged by TMA bulk-tensor
    copies (2) -- run the same per-point sums in the same order: identical
    images, on golden operators (offset and angle apertures, 3-D, user
    tables, tails of partial CTAs) and the 100 x 200 grid, float32 and bf16
    weights; no bounded wait gives up."""
    import torch

    from pylops_gb300.waveeqprocessing import Kirchhoff

    if case.startswith("grid"):
        c = _grid_100x200(dynamic=True, angleaperture=60.0 if case == "grid_60" else 30.0,
                          aperture=None if case == "grid_60" else 1.5)
        K = Kirchhoff(c["z"], c["x"], c["t"], c["srcs"], c["recs"], c["vel"], c["wav"], c["wc"], mode="analytic",
                      dynamic=True, angleaperture=c["angleaperture"], aperture=c["aperture"], engine="cuda",
                      dtype="float32")
    else:
        K = _op(load(case))
    if bf16:
        K.set_weight_precision("bfloat16")
    assert K.info()["adjoint_variant"] == 0  # the default
    d = torch.as_tensor(np.random.default_rng(4).standard_normal(K.shape[0]).astype(np.float32), device="cuda")
    out = []
    for v in (0, 1, 2, 0):
        K.set_adjoint_variant(v)
        assert K.info()["adjoint_variant"] == v
        out.append((K.H @ d).cpu().numpy())
    assert all(np.array_equal(out[0], a) for a in out[1:])
    assert K.info()["wait_error"] == 0