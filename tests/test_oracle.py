"""The FP64 oracle against golden vectors produced by the reference itself."""

import os

import numpy as np
import pytest

from oracle import kirchhoff_oracle as ko
from tests.conftest import GOLDEN

CASES = ["k2d_kin", "k2d_dyn_ap", "k2d_dyn_noap", "k3d_kin", "k3d_dyn", "k2d_dyn_byot", "k2d_kin_f32",
         "k2d_wavfilter", "k3d_wavfilter"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def build(g):
    y = g.get("y")
    kw = dict(y=y)
    if "vel_model" in g:
        vel = g["vel_model"]
        kw.update(mode="byot", trav=(g["trav_in_srcs"], g["trav_in_recs"]),
                  amp=(g["amp_in_srcs"], g["amp_in_recs"]))
    else:
        vel = float(g["vel_scalar"])
        kw.update(mode="analytic")
    if "aperture_in" in g:
        kw["aperture"] = float(g["aperture_in"])
    if "angleaperture_in" in g:
        kw["angleaperture"] = float(g["angleaperture_in"])
    elif bool(g["dynamic"]):
        kw["angleaperture"] = None if np.allclose(g["angleaperture"], np.deg2rad([0.0, 1000.0])) else 90.0
    wav = g["wav"]
    if "wavfilter_in" in g:  # the golden's wav is the reshaped one
        kw["wavfilter"] = True
        wav = g["wav_in"]
    return ko.KirchhoffOracle(g["z"], g["x"], g["t"], g["srcs"], g["recs"], vel, wav,
                              int(g["wavc"]), dynamic=bool(g["dynamic"]), **kw)


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_tables_match_reference(name):
    g = load(name)
    K = build(g)
    np.testing.assert_allclose(K.trav_srcs, g["trav_srcs"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(K.trav_recs, g["trav_recs"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(K.aperture, g["aperture"])
    np.testing.assert_allclose(K.angleaperture, g["angleaperture"])
    np.testing.assert_allclose(K.aperturetap, g["aperturetap"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(K.wav, g["wav"], rtol=1e-12, atol=1e-14)
    if K.dynamic:
        for k in ("amp_srcs", "amp_recs", "angle_srcs", "angle_recs", "vel"):
            np.testing.assert_allclose(getattr(K, k), g[k], rtol=1e-12, atol=1e-14, err_msg=k)
        np.testing.assert_array_equal(K.six, g["six"])
        np.testing.assert_array_equal(K.rix, g["rix"])


@pytest.mark.parametrize("name", CASES)
def test_spread_gather_match_reference(name):
    g = load(name)
    K = build(g)
    tol = 1e-6 if g["fwd"].dtype == np.float32 or g["spread"].dtype == np.float32 else 1e-12
    assert rel(K.spread(g["m_in"]), g["spread"]) < tol
    assert rel(K.gather(g["d_in"]), g["gather"]) < max(tol, 1e-12)


@pytest.mark.parametrize("name", CASES)
def test_matvec_rmatvec_match_reference(name):
    g = load(name)
    K = build(g)
    tol = 1e-6 if g["adj"].dtype == np.float32 else 1e-11
    assert rel(K.matvec(g["m_in"]), g["fwd"]) < tol
    assert rel(K.rmatvec(g["d_in"]), g["adj"]) < tol


def test_convolve1d_matches_reference():
    g = load("convolve1d")
    keys = sorted(k[2:] for k in g if k.startswith("h_"))
    assert len(keys) == 6
    for key in keys:
        nh, off = map(int, key.split("_"))
        h = ko.pad_wavelet(g["h_" + key], off)
        x = g["x_" + key]
        np.testing.assert_allclose(ko.conv_same(x, h), g["fwd_" + key], rtol=1e-9, atol=1e-10, err_msg=key)
        np.testing.assert_allclose(ko.conv_same(x, h[::-1].copy()), g["adj_" + key], rtol=1e-9, atol=1e-10, err_msg=key)


def test_solvers_match_reference():
    g = load("solvers")
    K = build(load("k2d_dyn_noap"))
    d = g["d"]
    out = ko.lsqr(K.matvec, K.rmatvec, d, K.ni, niter=12)
    assert out[1] == int(g["lsqr_istop"]) and out[2] == int(g["lsqr_iiter"])
    np.testing.assert_allclose(out[9], g["lsqr_cost"], rtol=1e-8)
    np.testing.assert_allclose(np.array(out[10]), g["lsqr_iterates"].reshape(len(out[10]), -1), rtol=1e-7, atol=1e-9)
    for k, i in (("lsqr_r1", 3), ("lsqr_r2", 4), ("lsqr_anorm", 5), ("lsqr_acond", 6), ("lsqr_arnorm", 7), ("lsqr_xnorm", 8)):
        np.testing.assert_allclose(out[i], g[k], rtol=1e-7, err_msg=k)
    out = ko.cgls(K.matvec, K.rmatvec, d, K.ni, niter=12, tol=1e-10)
    np.testing.assert_allclose(out[5], g["cgls_cost"], rtol=1e-8)
    np.testing.assert_allclose(np.array(out[6]), g["cgls_iterates"].reshape(len(out[6]), -1), rtol=1e-7, atol=1e-9)
    out = ko.lsqr(K.matvec, K.rmatvec, d, K.ni, niter=6, damp=0.1)
    np.testing.assert_allclose(out[9], g["lsqrd_cost"], rtol=1e-8)
    np.testing.assert_allclose(out[0], g["lsqrd_x"].ravel(), rtol=1e-7, atol=1e-9)
    out = ko.cgls(K.matvec, K.rmatvec, d, K.ni, niter=6, damp=0.1, tol=1e-10, x0=0.1 * np.ones(K.ni))
    np.testing.assert_allclose(out[5], g["cglsd_cost"], rtol=1e-8)
    np.testing.assert_allclose(out[0], g["cglsd_x"].ravel(), rtol=1e-7, atol=1e-9)


def test_traveltime_known_answer():
    g = load("traveltime_ana")
    src = np.array([100, 0])[:, np.newaxis]
    ts, tr, ds, dr, _, _ = ko.traveltime_table_analytic(np.arange(0, 200, 1), np.arange(0, 200, 1), src, src, 500.0)
    assert ts[0, 0] == 100 / 500.0 == float(g["trav00"])
    assert ds[0, 0] + dr[0, 0] == 200 == float(g["dist00"])


@pytest.mark.parametrize("name", CASES)
def test_c_oracle_matches_reference(name):
    """The OpenMP C restatement against the same golden vectors."""
    from oracle.kirch_oracle_c import COracle

    g = load(name)
    K = build(g)
    C = COracle(K, K.h)
    tol = 1e-6 if g["adj"].dtype == np.float32 else 1e-11
    assert rel(C.spread(g["m_in"]), g["spread"]) < max(tol, 1e-12)
    assert rel(C.gather(g["d_in"]), g["gather"]) < max(tol, 1e-12)
    assert rel(C.matvec(g["m_in"]), g["fwd"]) < tol
    assert rel(C.rmatvec(g["d_in"]), g["adj"]) < tol


@pytest.mark.parametrize("name", ["k2d_single", "k2d_single_neg"])
def test_single_table_oracle_matches_reference(name):
    """mode='byot' with one (ni, ns*nr) table: index/fraction, spreading,
    gathering and the full operator with the wavelet."""
    from oracle.kirchhoff_oracle import (conv_same, pad_wavelet, single_table_index, trav_matvec,
                                         trav_rmatvec)

    g = load(name)
    nsnr, nt, ni = int(g["ns"]) * int(g["nr"]), int(g["nt"]), int(g["ni"])
    it, w = single_table_index(g["trav_table"], float(g["dt"]))
    assert np.array_equal(it, g["itrav"])
    np.testing.assert_allclose(w, g["travd"], rtol=0, atol=1e-12)
    if name.endswith("neg"):
        assert np.any((it == 0) & (w < 0)), "negative-time quirk not exercised"
    y = trav_matvec(g["m_in"], nsnr, nt, ni, it, w)
    assert rel(y, g["spread"]) < 1e-12
    img = trav_rmatvec(g["d_in"], nsnr, nt, ni, it, w)
    assert rel(img, g["gather"]) < 1e-12
    h = pad_wavelet(g["wav"], int(g["wavc"]))
    assert rel(conv_same(y, h).ravel(), g["fwd"]) < 1e-10
    dc = conv_same(np.asarray(g["d_in"]).reshape(nsnr, nt), h[::-1].copy())
    assert rel(trav_rmatvec(dc, nsnr, nt, ni, it, w), g["adj"]) < 1e-10


def test_nsconv2d_oracle_matches_reference():
    from oracle.nsconv2d_oracle import nsconv2d

    g = load("nsconv2d")
    assert rel(nsconv2d(g["x_in"], g["hs"], g["ihx"], g["ihz"]), g["fwd"]) < 1e-12
    assert rel(nsconv2d(g["y_in"], g["hs"], g["ihx"], g["ihz"], adjoint=True), g["adj"]) < 1e-12


def test_eikonal_oracle_matches_analytic_and_the_package_solver():
    """The oracle's fast-marching tables (oracle/eikonal_oracle.c): within
    the reference's analytic-vs-eikonal bar (test_kirchhoff.py:163-212,
    decimal=2) at constant velocity, and equal to the package's own
    fast-marching solver on a variable-velocity 2-D and 3-D grid (two
    independent restatements of the same method; tolerance 1e-12)."""
    from oracle.kirchhoff_oracle import traveltime_table_analytic, traveltime_table_eikonal
    from pylops_gb300.waveeqprocessing.kirchhoff import Kirchhoff

    z = np.arange(20) * 2.0
    x = np.arange(12) * 1.0
    s = np.vstack((np.linspace(0, 11, 6), 2 * np.ones(6)))
    r = np.vstack((np.linspace(0, 11, 2), 2 * np.ones(2)))
    te = traveltime_table_eikonal(z, x, s, r, 500 * np.ones((12, 20)))
    ta = traveltime_table_analytic(z, x, s, r, 500.0)
    np.testing.assert_array_almost_equal(ta[0], te[0], decimal=2)
    np.testing.assert_array_almost_equal(ta[1], te[1], decimal=2)

    rng = np.random.default_rng(0)
    z = np.arange(40) * 5.0
    x = np.arange(50) * 5.0
    X, Z = np.meshgrid(x, z, indexing="ij")
    vel = 1500 + 0.5 * Z + 200 * np.exp(-((X - 120) ** 2 + (Z - 100) ** 2) / (2 * 30.0 ** 2))
    s = np.vstack((np.linspace(x[0], x[-1], 5), np.zeros(5)))
    r = np.vstack((np.linspace(x[0], x[-1], 7), np.full(7, 10.0)))
    a = traveltime_table_eikonal(z, x, s, r, vel)
    b = Kirchhoff._traveltime_table(z, x, s, r, vel, mode="eikonal")
    for i in range(4):
        np.testing.assert_allclose(a[i], b[i], rtol=1e-12, atol=0)
    for i in (4, 5):
        for k in range(2):
            np.testing.assert_allclose(a[i][k], b[i][k], rtol=1e-9, atol=1e-15)

    y = np.arange(8) * 10.0
    z = np.arange(9) * 10.0
    x = np.arange(10) * 10.0
    v3 = 2000 + 300 * rng.random((8, 10, 9))
    s3 = np.vstack(([20.0, 50.0], [30.0, 60.0], [0.0, 0.0]))
    r3 = np.vstack(([0.0, 70.0], [10.0, 90.0], [0.0, 0.0]))
    a = traveltime_table_eikonal(z, x, s3, r3, v3, y=y)
    b = Kirchhoff._traveltime_table(z, x, s3, r3, v3, y=y, mode="eikonal")
    for i in range(4):
        np.testing.assert_allclose(a[i], b[i], rtol=1e-12, atol=0)


def test_unit_speed_fast_marching_tables_are_shifts_of_one_corner_table():
    """The premise of the device distance rows: with unit speed a point's
    fast-marching table depends only on the offset from the point, so every
    distance row is the table of a point at the grid's corner read at
    (|ix - px|, |iz - pz|).  Held bit for bit with the oracle's fast
    marching (kirchhoff.py:609-638 computes the distances with
    skfmm.distance) on an anisotropic grid, points on edges, corners and
    inside."""
    from oracle.kirch_oracle_c import eikonal_tables

    nx, nz, hx, hz = 37, 23, 5.0, 4.0
    pts = np.array([[0, 0], [36, 22], [18, 0], [0, 11], [7, 13], [36, 0], [20, 21]], np.int32)
    _, own = eikonal_tables((nx, nz), (hx, hz), 1.0, pts, with_trav=False)
    _, corner = eikonal_tables((nx, nz), (hx, hz), 1.0, np.array([[0, 0]], np.int32), with_trav=False)
    corner = corner[:, 0].reshape(nx, nz)
    I0, I1 = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    for k, (p0, p1) in enumerate(pts):
        shifted = corner[np.abs(I0 - p0), np.abs(I1 - p1)].ravel()
        assert np.array_equal(shifted, own[:, k]), (p0, p1)
