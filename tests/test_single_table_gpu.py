"""Single traveltime table (mode='byot' with trav of shape (ni, ns*nr),
kirchhoff.py:396-398, 684-725) on the GPU against the reference's golden
vectors (non-negative times, and times shifted negative to exercise the
truncation quirk) and, at a larger size, against the float64 oracle.
Tolerance 1e-5 relative L2 (float32 against float64)."""

import numpy as np
import pytest

from tests.helpers import load, rel

pytestmark = pytest.mark.gpu


def _op(g, dtype="float32", table=None):
    from pylops_gb300.waveeqprocessing import Kirchhoff

    return Kirchhoff(g["z"], g["x"], g["t"], g["srcs"], g["recs"], float(g["vel_scalar"]), g["wav"], int(g["wavc"]),
                     mode="byot", trav=g["trav_table"] if table is None else table, engine="cuda", dtype=dtype)


@pytest.mark.parametrize("name", ["k2d_single", "k2d_single_neg"])
def test_single_table_matches_reference(name):
    g = load(name)
    K = _op(g)
    assert not K.travsrcrec
    assert np.array_equal(K.itrav, g["itrav"])
    assert rel(K @ g["m_in"], g["fwd"]) < 1e-5
    assert rel(K.H @ g["d_in"], g["adj"]) < 1e-5
    assert rel(K.spread(g["m_in"]), g["spread"]) < 1e-5
    assert rel(K.gather(g["d_in"]), g["gather"]) < 1e-5


def test_single_table_dottest_determinism_and_reassignment():
    import torch

    from pylops_gb300.utils.dottest import dottest

    g = load("k2d_single")
    K = _op(g)
    assert dottest(K, *K.shape, rtol=1e-4)
    m = torch.randn(K.ni, device="cuda")
    a, b = K @ m, K @ m
    assert torch.equal(a, b)
    d = torch.randn(K.shape[0], device="cuda")
    assert torch.equal(K.H @ d, K.H @ d)
    # reassigning the table refreshes the device copy
    K.trav = g["trav_table"] * 1.1
    K2 = _op(g, table=g["trav_table"] * 1.1)
    assert rel((K @ g["m_in"]), (K2 @ g["m_in"])) < 1e-7


def test_single_table_dynamic_raises_like_reference():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    g = load("k2d_single")
    with pytest.raises(NotImplementedError):
        Kirchhoff(g["z"], g["x"], g["t"], g["srcs"], g["recs"], 500.0, g["wav"], int(g["wavc"]), mode="byot",
                  trav=g["trav_table"], dynamic=True, amp=g["trav_table"], engine="cuda")


@pytest.mark.parametrize("nx,nz", [(300, 200), (301, 199)])
def test_single_table_medium_size_against_oracle(nx, nz):
    """300 x 200 image (an odd-sized one too: the scalar gather), 16 x 64
    traces, nt = 700: a 245 MB table; both forward variants."""
    from oracle.kirchhoff_oracle import conv_same, pad_wavelet, single_table_index, trav_matvec, trav_rmatvec
    from pylops_gb300.utils.wavelets import ricker
    from pylops_gb300.waveeqprocessing import Kirchhoff

    nt, dt = 700, 0.002
    z, x, t = np.arange(nz) * 5.0, np.arange(nx) * 5.0, np.arange(nt) * dt
    ns, nr = 16, 64
    srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
    recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
    X, Z = np.meshgrid(x, z, indexing="ij")
    v = 1500.0 + 0.5 * Z.ravel()
    ds = np.sqrt((X.ravel()[:, None] - srcs[0][None]) ** 2 + Z.ravel()[:, None] ** 2)
    dr = np.sqrt((X.ravel()[:, None] - recs[0][None]) ** 2 + Z.ravel()[:, None] ** 2)
    table = ((ds[:, :, None] + dr[:, None, :]) / v[:, None, None]).reshape(nx * nz, ns * nr)
    wav, _, wc = ricker(t[:41], f0=15)
    K = Kirchhoff(z, x, t, srcs, recs, 1500.0, wav, wc, mode="byot", trav=table, engine="cuda", dtype="float32")
    rng = np.random.default_rng(0)
    m = rng.standard_normal(K.ni)
    d = rng.standard_normal(K.shape[0])
    it, w = single_table_index(table, dt)
    h = pad_wavelet(wav, wc)
    yo = conv_same(trav_matvec(m, ns * nr, nt, K.ni, it, w), h).ravel()
    for variant in (0, 1):
        K.set_spread_variant(variant)
        assert rel(K @ m.astype(np.float32), yo) < 1e-5, variant
    io = trav_rmatvec(conv_same(d.reshape(ns * nr, nt), h[::-1].copy()), ns * nr, nt, K.ni, it, w)
    assert rel(K.H @ d.astype(np.float32), io) < 1e-5
