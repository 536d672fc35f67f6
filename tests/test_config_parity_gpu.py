"""Parity on the workload configurations themselves, against the float64
oracle on identical inputs:

* the 100 x 200 analytic kinematic workload (10 x 50 traces, nt = 651):
  10 LSQR iterations, iterate by iterate (cls_basic.py:835-1136);
* the 300 x 800 eikonal dynamic workload with 4 of its 64 sources (all 400
  receivers): the 30-iteration LSQR residual history;
* the batched workload: the block-diagonal batch operator on uneven
  problems, each block against the oracle;
* the fixed-point traveltime index decisions at the 300 x 800 workload,
  counted against float64 int(t/dt).

Tolerances: the operator is float32 (forward/adjoint 1e-5 relative L2
against float64); LSQR keeps float32 vectors and float64 scalars while the
oracle keeps float64 vectors.  On the kinematic 100 x 200 problem (20,000
unknowns, 500 traces, strongly ill-conditioned) the iterates agree to 1e-4
over the first 8 iterations; from there LSQR reaches the small singular
values, where the float32 operator's rounding (1e-7 per application) is
amplified: measured 4e-4 at iteration 8 and 6e-3 at iteration 9, so the
last two are held to 2e-2.  The residual history agrees to 1e-7 over
iterations 0-8 (held to 1e-5) and then by 1e-4 and 1e-2 (held to 2e-2).
The 30-iteration history of the 300 x 800 problem is held to 1e-3.
"""

import numpy as np
import pytest

from oracle import kirchhoff_oracle as ko
from tests.helpers import rel

pytestmark = pytest.mark.gpu


def _config1():
    """100 x 200 grid at 4 m, v = 2000 m/s, 10 sources and 50 receivers at
    z = 0, nt = 651 at 4 ms, 20 Hz Ricker; reflectivity of 3 horizontal and
    one 10-degree dipping reflector with N(0,1) amplitudes (seed 0)."""
    nz, nx, ns, nr, nt = 100, 200, 10, 50, 651
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
    a = rng.standard_normal()
    for ix in range(nx):
        iz = int(round(10 + ix * np.tan(np.deg2rad(10.0))))
        if iz < nz:
            refl[ix, iz] += a
    return (z, x, t, srcs, recs, 2000.0, wav, wc), refl.ravel()


def test_config1_lsqr_tracks_oracle_iterates():
    from oracle.kirch_oracle_c import COracle, build
    from pylops_gb300.optimization import lsqr
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, refl = _config1()
    K = Kirchhoff(*args, mode="analytic", engine="cuda", dtype="float32")
    O = ko.KirchhoffOracle(*args, mode="analytic")
    build()
    C = COracle(O, O.h)
    d = C.matvec(refl)
    # forward, adjoint and dottest at this size
    assert rel(K @ refl.astype(np.float32), d) < 1e-5
    assert rel(K.H @ d.astype(np.float32), C.rmatvec(d)) < 1e-5
    its = []
    out = lsqr(K, d.astype(np.float32), niter=10, callback=lambda x: its.append(np.array(x, np.float64)))
    ref = ko.lsqr(C.matvec, C.rmatvec, d, K.ni, niter=10)
    assert out[2] == ref[2] == 10
    assert len(its) == len(ref[10]) == 10
    for k in range(10):
        assert rel(its[k], ref[10][k]) < (1e-4 if k < 8 else 2e-2), (k, rel(its[k], ref[10][k]))
    np.testing.assert_allclose(out[-1][:9], ref[9][:9], rtol=1e-5)
    np.testing.assert_allclose(out[-1][9:], ref[9][9:], rtol=2e-2)
    # the graph path (one launch for the 10 iterations) gives the same iterate
    g = lsqr(K, d.astype(np.float32), niter=10)
    assert np.array_equal(g[0], out[0])


def test_config2_lsqr_history_reduced_sources():
    """The 300 x 800 eikonal dynamic workload (60-degree angle aperture) with
    4 of its 64 sources; the oracle gets the operator's own float64 tables."""
    import torch

    from bench import build_operator, make_workload, subset_sources
    from oracle.kirch_oracle_c import COracle, build
    from pylops_gb300.optimization.cls_basic import LSQR

    w = subset_sources(make_workload(), 4)
    K, _ = build_operator(w)
    build()
    C = COracle(K, ko.pad_wavelet(np.asarray(K.wav), K.wavcenter))
    refl = np.asarray(w["refl"], np.float64).ravel()
    d = C.matvec(refl)
    dg = torch.as_tensor(d.astype(np.float32), device="cuda")
    out = LSQR(K).solve(dg, niter=30, atol=0.0, btol=0.0, calc_var=False)
    ref = ko.lsqr(C.matvec, C.rmatvec, d, K.ni, niter=30, atol=0.0, btol=0.0)
    assert int(out[2]) == ref[2] == 30
    cost = np.asarray(out[-1], np.float64)
    np.testing.assert_allclose(cost, ref[9], rtol=1e-3)
    assert rel(out[0].cpu().numpy(), ref[0]) < 1e-3


def test_batch_blocks_match_oracle_on_uneven_problems():
    from pylops_gb300.waveeqprocessing.batch import build_batch, random_problems

    probs = random_problems(3, seed=21, nt=301)
    sizes = {(len(p["z"]), len(p["x"]), p["srcs"].shape[1], p["recs"].shape[1]) for p in probs}
    assert len(sizes) == 3  # uneven grids and shot counts
    B = build_batch(probs)
    rng = np.random.default_rng(1)
    m = rng.standard_normal(B.shape[1])
    d = rng.standard_normal(B.shape[0])
    for R in (2, 8):
        B.set_tile(R)
        y = B @ m.astype(np.float32)
        x = B.H @ d.astype(np.float32)
        for p, mp, dp, yp, xp in zip(probs, B.split_model(m), B.split_data(d), B.split_data(y),
                                     B.split_model(x)):
            O = ko.KirchhoffOracle(p["z"], p["x"], p["t"], p["srcs"], p["recs"], p["vel"], p["wav"],
                                   p["wavcenter"], mode="analytic")
            assert rel(yp, O.matvec(np.asarray(mp))) < 1e-5
            assert rel(xp, O.rmatvec(np.asarray(dp))) < 1e-5


def test_fixed_point_index_decisions_at_the_300x800_workload():
    """Count the pair-points whose fixed-point time index differs from the
    reference's float64 int((ts + tr)/dt), on 4 sources x 400 receivers of
    the 300 x 800 workload (3.8e8 pair-points).  Such a point sits within
    2^-frac_bits samples of a bin edge, where the linear interpolation is
    continuous, so its contribution differs by at most that fraction."""
    from bench import build_operator, make_workload, subset_sources

    w = subset_sources(make_workload(), 4)
    K, _ = build_operator(w)
    F = K.info()["frac_bits"]
    ts, tr = np.asarray(K.trav_srcs), np.asarray(K.trav_recs)
    inv_dt = 1.0 / K.dt  # the quantisation of the table upload: rint(t * (1/dt) * 2^F)
    qs = np.rint(ts * inv_dt * 2.0 ** F).astype(np.int64)
    qr = np.rint(tr * inv_dt * 2.0 ** F).astype(np.int64)
    differ = total = 0
    for isrc in range(K.ns):
        t = ts[:, isrc:isrc + 1] + tr
        it_ref = (t / K.dt).astype(np.int64)
        it_fix = (qs[:, isrc:isrc + 1] + qr) >> F
        valid = (it_ref >= 0) & (it_ref < K.nt - 1)
        differ += int(np.count_nonzero((it_ref != it_fix) & valid))
        total += int(np.count_nonzero(valid))
    frac = differ / total
    print(f"fixed-point index decisions that differ: {differ} of {total} ({frac:.2e}), F = {F}")
    assert frac < 1e-4
