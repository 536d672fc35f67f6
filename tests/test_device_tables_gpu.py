"""Tables built on the device (kgb_kirchhoff_build_tables) against the host
construction of the same operator (tables='host': numpy tables as the
reference builds them, kirchhoff.py:303-393, 503-657, and the package's
host fast-marching solver for eikonal tables).

Tolerances: analytic traveltimes, distances and amplitudes are the same
float64 operations in the same order, so they are held to equality; angles
go through atan2/acos, whose last bit may differ between the device and the
host library, so they are held to 1e-12 radians; the operators' outputs to
1e-6 relative (a last-bit angle difference can move a float32 weight by one
ulp).  Eikonal tables come from the same fast-marching equations solved by
sweeping instead of marching: most values are equal, and where the marching
order picked another upwind stencil they differ by at most ~3e-5 of the
largest time (measured on CPU emulations of both); held to 1e-4 relative
against the host solver, and to the reference's own analytic-vs-eikonal bar
(decimal=2, test_kirchhoff.py:163-212).
"""

import numpy as np
import pytest

from tests.helpers import rel

pytestmark = pytest.mark.gpu


def _ops(args, **kw):
    from pylops_gb300.waveeqprocessing import Kirchhoff

    Kd = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    Kh = Kirchhoff(*args, engine="cuda", dtype="float32", tables="host", **kw)
    return Kd, Kh


def _geometry2d(nz=40, nx=60, ns=5, nr=9, nt=300, dz=4.0, dx=5.0, zs=0.0):
    from oracle.kirchhoff_oracle import ricker

    z = np.arange(nz) * dz
    x = np.arange(nx) * dx
    t = np.arange(nt) * 0.002
    srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.full(ns, zs)))
    recs = np.vstack((np.linspace(x[3], x[-4], nr), np.full(nr, zs + dz)))
    wav, _, wc = ricker(t[:31], f0=25)
    return z, x, t, srcs, recs, wav, wc


@pytest.mark.parametrize("dynamic", [False, True])
def test_analytic_2d_tables_equal_host_tables(dynamic):
    z, x, t, srcs, recs, wav, wc = _geometry2d()
    kw = dict(mode="analytic", dynamic=dynamic, angleaperture=50.0 if dynamic else 90.0,
              aperture=3.0 if dynamic else None)
    Kd, Kh = _ops((z, x, t, srcs, recs, 1800.0, wav, wc), **kw)
    assert np.array_equal(Kd.trav_srcs, Kh.trav_srcs) and np.array_equal(Kd.trav_recs, Kh.trav_recs)
    if dynamic:
        assert Kd.maxdist == Kh.maxdist
        assert np.array_equal(Kd.amp_srcs, Kh.amp_srcs) and np.array_equal(Kd.amp_recs, Kh.amp_recs)
        assert np.max(np.abs(Kd.angle_srcs - Kh.angle_srcs)) < 1e-12
        assert np.max(np.abs(Kd.angle_recs - Kh.angle_recs)) < 1e-12
    rng = np.random.default_rng(0)
    m = rng.standard_normal(Kd.ni).astype(np.float32)
    d = rng.standard_normal(Kd.shape[0]).astype(np.float32)
    assert rel(Kd @ m, Kh @ m) < 1e-6
    assert rel(Kd.H @ d, Kh.H @ d) < 1e-6


def test_analytic_3d_tables_equal_host_tables():
    from oracle.kirchhoff_oracle import ricker

    y, x, z = np.arange(6) * 10.0, np.arange(8) * 10.0, np.arange(12) * 10.0
    t = np.arange(200) * 0.004
    sy, sx = np.meshgrid([10.0, 40.0], [20.0, 50.0], indexing="ij")
    ry, rx = np.meshgrid([0.0, 30.0], [10.0, 60.0], indexing="ij")
    srcs = np.vstack((sy.ravel(), sx.ravel(), np.zeros(4)))
    recs = np.vstack((ry.ravel(), rx.ravel(), np.zeros(4)))
    wav, _, wc = ricker(t[:21], f0=20)
    for dynamic in (False, True):
        Kd, Kh = _ops((z, x, t, srcs, recs, 2500.0, wav, wc), y=y, mode="analytic", dynamic=dynamic,
                      angleaperture=60.0)
        assert np.array_equal(Kd.trav_srcs, Kh.trav_srcs) and np.array_equal(Kd.trav_recs, Kh.trav_recs)
        if dynamic:
            assert np.array_equal(Kd.amp_srcs, Kh.amp_srcs)
            # ns == nr: receiver angles take the source table's x-gradient sign
            assert np.max(np.abs(Kd.angle_recs - Kh.angle_recs)) < 1e-12
        m = np.random.default_rng(1).standard_normal(Kd.ni).astype(np.float32)
        assert rel(Kd @ m, Kh @ m) < 1e-6


def test_eikonal_2d_tables_match_host_fast_marching():
    import time

    z, x, t, srcs, recs, wav, wc = _geometry2d(nz=70, nx=90, ns=6, nr=11)
    X, Z = np.meshgrid(x, z, indexing="ij")
    vel = 1500.0 + 0.6 * Z + 250.0 * np.exp(-((X - 200.0) ** 2 + (Z - 150.0) ** 2) / (2 * 40.0 ** 2))
    t0 = time.perf_counter()
    Kd, Kh = _ops((z, x, t, srcs, recs, vel, wav, wc), mode="eikonal", dynamic=True, angleaperture=60.0)
    for a, b in ((Kd.trav_srcs, Kh.trav_srcs), (Kd.trav_recs, Kh.trav_recs), (Kd.amp_srcs, Kh.amp_srcs)):
        err = np.max(np.abs(a - b) / np.abs(b).max())
        print(f"device eikonal vs host fast marching: max rel diff {err:.2e}")
        assert err < 1e-4, err
    rng = np.random.default_rng(2)
    m = rng.standard_normal(Kd.ni).astype(np.float32)
    assert rel(Kd @ m, Kh @ m) < 1e-3
    print(f"two operators built in {time.perf_counter() - t0:.2f} s")


def test_eikonal_device_tables_match_analytic_decimal2():
    """The reference's test_traveltime_table check (decimal=2) with device
    eikonal tables in a homogeneous model."""
    from pylops_gb300.waveeqprocessing import Kirchhoff

    z = np.arange(20) * 2.0
    x = np.arange(12) * 1.0
    t = np.arange(50) * 0.004
    s = np.vstack((np.linspace(0, 11, 6), 2 * np.ones(6)))
    r = np.vstack((np.linspace(0, 11, 2), 2 * np.ones(2)))
    wav = np.array([0.0, 1.0, 0.0])
    Ke = Kirchhoff(z, x, t, s, r, 500 * np.ones((12, 20)), wav, 1, mode="eikonal", engine="cuda")
    Ka = Kirchhoff(z, x, t, s, r, 500.0, wav, 1, mode="analytic", engine="cuda")
    np.testing.assert_array_almost_equal(Ka.trav_srcs, Ke.trav_srcs, decimal=2)
    np.testing.assert_array_almost_equal(Ka.trav_recs, Ke.trav_recs, decimal=2)


def test_reassigned_tables_after_device_build():
    """Reassigning a table attribute of a device-built operator re-uploads
    it, as for host-built tables (test_kirchhoff.py:252-258)."""
    z, x, t, srcs, recs, wav, wc = _geometry2d()
    Kd, Kh = _ops((z, x, t, srcs, recs, 1800.0, wav, wc), mode="analytic", dynamic=True, angleaperture=50.0)
    Kd.trav_srcs = Kh.trav_srcs * 1.05
    Kh.trav_srcs = Kh.trav_srcs * 1.05
    Kd.amp_recs = Kh.amp_recs * 2.0
    Kh.amp_recs = Kh.amp_recs * 2.0
    m = np.random.default_rng(3).standard_normal(Kd.ni).astype(np.float32)
    assert rel(Kd @ m, Kh @ m) < 1e-6


def test_eikonal_3d_tables_match_host_fast_marching():
    """3-D eikonal tables by sweeping the 8 diagonal orders on the device
    against the host fast-marching solver (tables='host'), heterogeneous
    velocity, sources and receivers on the surface and one buried point."""
    from oracle.kirchhoff_oracle import ricker

    y, x, z = np.arange(10) * 10.0, np.arange(14) * 8.0, np.arange(18) * 5.0
    Y, X, Z = np.meshgrid(y, x, z, indexing="ij")
    vel = 1500.0 + 0.8 * Z + 300.0 * np.exp(-((X - 50.0) ** 2 + (Y - 40.0) ** 2 + (Z - 45.0) ** 2) / (2 * 25.0 ** 2))
    t = np.arange(150) * 0.002
    sy, sx = np.meshgrid([10.0, 60.0], [16.0, 80.0], indexing="ij")
    ry, rx = np.meshgrid([0.0, 40.0, 90.0], [8.0, 56.0, 104.0], indexing="ij")
    srcs = np.vstack((np.append(sy.ravel(), 50.0), np.append(sx.ravel(), 48.0), np.append(np.zeros(4), 30.0)))
    recs = np.vstack((ry.ravel(), rx.ravel(), np.zeros(9)))
    wav, _, wc = ricker(t[:21], f0=20)
    Kd, Kh = _ops((z, x, t, srcs, recs, vel, wav, wc), y=y, mode="eikonal", dynamic=True, angleaperture=70.0)
    for a, b in ((Kd.trav_srcs, Kh.trav_srcs), (Kd.trav_recs, Kh.trav_recs), (Kd.amp_srcs, Kh.amp_srcs),
                 (Kd.amp_recs, Kh.amp_recs)):
        err = np.max(np.abs(a - b) / np.abs(b).max())
        print(f"3-D device eikonal vs host fast marching: max rel diff {err:.2e}")
        assert err < 1e-4, err
    m = np.random.default_rng(4).standard_normal(Kd.ni).astype(np.float32)
    assert rel(Kd @ m, Kh @ m) < 1e-3
