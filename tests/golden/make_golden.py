"""Generate golden input/output vectors from the PyLops reference itself.

Run where the reference (PyLops) source tree is available, with its
location in the environment variable PYLOPS_REFERENCE:

    PYLOPS_REFERENCE=<path to the PyLops source tree> python tests/golden/make_golden.py

It writes ``tests/golden/*.npz``.  Every case is built with the reference's
own public API (``pylops.waveeqprocessing.Kirchhoff`` with ``engine='numpy'``,
which is the same Python source the ``numba`` engine JIT-compiles,
``pylops.optimization.basic.lsqr/cgls`` and ``Convolve1D``) on seeded inputs,
so the fixtures pin both the oracle and the CUDA path without the reference
being present at test time.
"""

import os
import sys
import warnings

import numpy as np

if os.environ.get("PYLOPS_REFERENCE"):
    sys.path.insert(0, os.environ["PYLOPS_REFERENCE"])

warnings.filterwarnings("ignore")

import pylops  # noqa: E402
from pylops.optimization.basic import cgls, lsqr  # noqa: E402
from pylops.signalprocessing import Convolve1D  # noqa: E402
from pylops.utils.wavelets import ricker  # noqa: E402
from pylops.waveeqprocessing.kirchhoff import Kirchhoff  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# Geometry of pytests/test_kirchhoff.py:22-65
PAR = dict(ny=3, nx=12, nz=20, nt=50, dy=3, dx=1, dz=2, dt=0.004, nsy=4, nry=3, nsx=6, nrx=2)
v0 = 500.0
y = np.arange(PAR["ny"]) * PAR["dy"]
x = np.arange(PAR["nx"]) * PAR["dx"]
z = np.arange(PAR["nz"]) * PAR["dz"]
t = np.arange(PAR["nt"]) * PAR["dt"]
sy = np.linspace(y.min(), y.max(), PAR["nsy"])
sx = np.linspace(x.min(), x.max(), PAR["nsx"])
syy, sxx = np.meshgrid(sy, sx, indexing="ij")
s2d = np.vstack((sx, 2 * np.ones(PAR["nsx"])))
s3d = np.vstack((syy.ravel(), sxx.ravel(), 2 * np.ones(PAR["nsx"] * PAR["nsy"])))
ry = np.linspace(y.min(), y.max(), PAR["nry"])
rx = np.linspace(x.min(), x.max(), PAR["nrx"])
ryy, rxx = np.meshgrid(ry, rx, indexing="ij")
r2d = np.vstack((rx, 2 * np.ones(PAR["nrx"])))
r3d = np.vstack((ryy.ravel(), rxx.ravel(), 2 * np.ones(PAR["nrx"] * PAR["nry"])))
wav, _, wavc = ricker(t[:21], f0=40)


def _save(name, K, xin, din, extra=None, geometry=None):
    fwd = np.asarray(K @ xin)
    adj = np.asarray(K.H @ din)
    rec = dict(
        ns=K.ns, nr=K.nr, nt=K.nt, ni=int(K.ni), dt=float(K.dt), nz=K.nz, nx=K.nx, ny=K.ny,
        ndims=K.ndims, dynamic=K.dynamic,
        trav_srcs=np.asarray(K.trav_srcs), trav_recs=np.asarray(K.trav_recs),
        m_in=xin, d_in=din, fwd=fwd, adj=adj,
        wav=np.asarray(K.wav), aperturetap=np.asarray(K.aperturetap),
        aperture=np.asarray(K.aperture, dtype=np.float64),
        angleaperture=np.asarray(K.angleaperture, dtype=np.float64),
        # intermediate: spreading without wavelet and gathering without wavelet
        spread=np.asarray(_spread_only(K, xin)), gather=np.asarray(_gather_only(K, din)),
    )
    if K.dynamic:
        rec.update(amp_srcs=np.asarray(K.amp_srcs), amp_recs=np.asarray(K.amp_recs),
                   angle_srcs=np.asarray(K.angle_srcs), angle_recs=np.asarray(K.angle_recs),
                   vel=np.asarray(K.vel), six=np.asarray(K.six), rix=np.asarray(K.rix))
    if geometry is not None:
        rec.update(geometry)
    if extra:
        rec.update(extra)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print("wrote", name, {k: np.shape(v) for k, v in rec.items() if np.ndim(v) > 0})


def _spread_only(K, xin):
    yy = np.zeros((K.nsnr, K.nt), dtype=K.dtype)
    return _call(K, K._kirch_matvec, xin.ravel(), yy)


def _gather_only(K, din):
    yy = np.zeros(K.ni, dtype=K.dtype)
    return _call(K, K._kirch_rmatvec, din.reshape(K.nsnr, K.nt), yy)


def _call(K, fn, a, b):
    if K.dynamic:
        return fn(a, b, K.ns, K.nr, K.nt, K.ni, K.dt, K.vel, K.trav_srcs, K.trav_recs,
                  K.amp_srcs, K.amp_recs, K.aperture[0], K.aperture[1], K.aperturetap,
                  K.nz, K.six, K.rix, K.angleaperture[0], K.angleaperture[1],
                  K.angle_srcs, K.angle_recs)
    return fn(a, b, K.ns, K.nr, K.nt, K.ni, K.dt, K.trav_srcs, K.trav_recs)


def geom2d():
    return dict(z=z, x=x, t=t, srcs=s2d, recs=r2d)


def geom3d():
    return dict(z=z, x=x, t=t, srcs=s3d, recs=r3d, y=y)


def main():
    rng = np.random.default_rng(1234)

    # 1) 2-D kinematic analytic, float64 (test_kirchhoff.py geometry)
    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=False, engine="numpy")
    _save("k2d_kin", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc), geometry=geom2d())

    # 2) 2-D dynamic analytic, angle aperture 20 deg (taper active), offset aperture 2.0
    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=True,
                  aperture=2.0, angleaperture=20.0, engine="numpy")
    _save("k2d_dyn_ap", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc, aperture_in=2.0, angleaperture_in=20.0), geometry=geom2d())

    # 3) 2-D dynamic analytic, no angle aperture
    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=True,
                  angleaperture=None, engine="numpy")
    _save("k2d_dyn_noap", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc), geometry=geom2d())

    # 4) 3-D kinematic analytic
    K = Kirchhoff(z, x, t, s3d, r3d, v0, wav, wavc, y=y, mode="analytic", dynamic=False, engine="numpy")
    _save("k3d_kin", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc), geometry=geom3d())

    # 5) 3-D dynamic analytic, angle aperture 45 deg.  The reference signs the
    # receiver angle with the source gradient (kirchhoff.py:386-393), which only
    # broadcasts when ns == nr, so this case uses 6 sources and 6 receivers.
    s3d6 = s3d[:, ::4].copy()
    K = Kirchhoff(z, x, t, s3d6, r3d, v0, wav, wavc, y=y, mode="analytic", dynamic=True,
                  angleaperture=45.0, engine="numpy")
    _save("k3d_dyn", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc, angleaperture_in=45.0),
          geometry=dict(z=z, x=x, t=t, srcs=s3d6, recs=r3d, y=y))
    # and record that ns != nr raises in the reference
    try:
        Kirchhoff(z, x, t, s3d, r3d, v0, wav, wavc, y=y, mode="analytic", dynamic=True, engine="numpy")
        raised = ""
    except ValueError as e:  # broadcast error
        raised = "ValueError: " + str(e)
    np.savez_compressed(os.path.join(OUT, "k3d_dyn_ns_ne_nr.npz"), raised=raised)

    # 6) 2-D dynamic byot with a heterogeneous velocity (tables from the analytic
    # constructor, scaled per image point so gradients/angles are non-trivial)
    ts, tr, ds, dr, _, _ = Kirchhoff._traveltime_table(z, x, s2d, r2d, v0, mode="analytic")
    scale = 1.0 + 0.3 * np.sin(np.arange(ts.shape[0]) / 7.0)[:, None]
    ts_b, tr_b = ts * scale, tr * scale
    as_b, ar_b = 1.0 / np.sqrt(ds + 1.0), 1.0 / np.sqrt(dr + 1.0)
    velm = v0 * (1.0 + 0.2 * rng.random((PAR["nx"], PAR["nz"])))
    K = Kirchhoff(z, x, t, s2d, r2d, velm, wav, wavc, mode="byot", dynamic=True,
                  trav=(ts_b, tr_b), amp=(as_b, ar_b), angleaperture=50.0, engine="numpy")
    _save("k2d_dyn_byot", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_model=velm, wavc=wavc, angleaperture_in=50.0,
                     trav_in_srcs=ts_b, trav_in_recs=tr_b, amp_in_srcs=as_b, amp_in_recs=ar_b),
          geometry=geom2d())

    # 7) float32 operator, reduced config-1-like geometry (constant velocity 2000 m/s,
    # 20 Hz Ricker on t[:41] -> 81 taps centred at 40, sources/receivers at z=0)
    nz1, nx1, nt1, dt1 = 30, 48, 160, 0.004
    z1 = np.arange(nz1) * 4.0
    x1 = np.arange(nx1) * 4.0
    t1 = np.arange(nt1) * dt1
    s1 = np.vstack((np.linspace(x1[0], x1[-1], 3), np.zeros(3)))
    r1 = np.vstack((np.linspace(x1[0], x1[-1], 8), np.zeros(8)))
    w1, _, wc1 = ricker(t1[:41], f0=20)
    K = Kirchhoff(z1, x1, t1, s1, r1, 2000.0, w1, wc1, mode="analytic", dynamic=False,
                  engine="numpy", dtype="float32")
    _save("k2d_kin_f32", K, rng.standard_normal(K.ni).astype(np.float32),
          rng.standard_normal(K.shape[0]).astype(np.float32),
          extra=dict(vel_scalar=2000.0, wavc=wc1),
          geometry=dict(z=z1, x=x1, t=t1, srcs=s1, recs=r1))

    # 8) Convolve1D impulse responses: odd and even filters, several offsets
    conv = {}
    for nh, off in [(81, 40), (81, 30), (21, 10), (20, 9), (20, 12), (7, 0)]:
        h = rng.standard_normal(nh)
        C = Convolve1D((5, 160), h=h, offset=off, axis=1)
        xin = rng.standard_normal((5, 160))
        conv[f"h_{nh}_{off}"] = h
        conv[f"x_{nh}_{off}"] = xin
        conv[f"fwd_{nh}_{off}"] = (C @ xin.ravel()).reshape(5, 160)
        conv[f"adj_{nh}_{off}"] = (C.H @ xin.ravel()).reshape(5, 160)
    np.savez_compressed(os.path.join(OUT, "convolve1d.npz"), **conv)
    print("wrote convolve1d")

    # 9) Solver iterates on a small Kirchhoff problem (LSQR and CGLS, reference classes)
    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=True,
                  angleaperture=None, engine="numpy")
    refl = np.zeros((PAR["nx"], PAR["nz"]))
    refl[:, PAR["nz"] // 2] = 1
    refl[:, 3 * PAR["nz"] // 4] = 1
    d = K @ refl.ravel()
    it_l, it_c = [], []
    out_l = lsqr(K, d, niter=12, damp=0.0, callback=lambda xx: it_l.append(np.array(xx).copy()))
    out_c = cgls(K, d, niter=12, damp=0.0, tol=1e-10, callback=lambda xx: it_c.append(np.array(xx).copy()))
    out_ld = lsqr(K, d, niter=6, damp=0.1)
    out_cd = cgls(K, d, x0=0.1 * np.ones(K.ni), niter=6, damp=0.1, tol=1e-10)
    np.savez_compressed(
        os.path.join(OUT, "solvers.npz"),
        refl=refl, d=d,
        lsqr_x=out_l[0], lsqr_istop=out_l[1], lsqr_iiter=out_l[2], lsqr_r1=out_l[3],
        lsqr_r2=out_l[4], lsqr_anorm=out_l[5], lsqr_acond=out_l[6], lsqr_arnorm=out_l[7],
        lsqr_xnorm=out_l[8], lsqr_cost=out_l[10], lsqr_iterates=np.array(it_l),
        cgls_x=out_c[0], cgls_istop=out_c[1], cgls_iiter=out_c[2], cgls_r1=out_c[3],
        cgls_r2=out_c[4], cgls_cost=out_c[5], cgls_iterates=np.array(it_c),
        lsqrd_x=out_ld[0], lsqrd_cost=out_ld[10], lsqrd_r1=out_ld[3], lsqrd_r2=out_ld[4],
        cglsd_x=out_cd[0], cglsd_cost=out_cd[5], cglsd_r1=out_cd[3], cglsd_r2=out_cd[4],
    )
    print("wrote solvers")

    # 10) known answers of test_kirchhoff.py:139-157
    src = np.array([100, 0])[:, np.newaxis]
    ta, tb, da, db, _, _ = Kirchhoff._traveltime_table(
        np.arange(0, 200, 1), np.arange(0, 200, 1), src, src, v0, mode="analytic")
    np.savez_compressed(os.path.join(OUT, "traveltime_ana.npz"),
                        trav00=ta[0, 0], dist00=da[0, 0] + db[0, 0], v0=v0,
                        pylops_version=str(pylops.__version__))
    print("wrote traveltime_ana")

    # 11) right-preconditioned LSQR with a warm start: lsqr(K * Diagonal(p), d, x0=z0)
    from pylops.basicoperators import Diagonal

    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=True,
                  angleaperture=None, engine="numpy")
    refl = np.zeros((PAR["nx"], PAR["nz"]))
    refl[:, PAR["nz"] // 2] = 1
    refl[:, 3 * PAR["nz"] // 4] = 1
    d = K @ refl.ravel()
    p = (1.0 + 0.1 * np.arange(PAR["nz"]))[np.newaxis, :] * np.ones((PAR["nx"], 1))
    z0 = 0.3 * refl.ravel() / p.ravel()
    its = []
    out = lsqr(K * Diagonal(p.ravel()), d, x0=z0, niter=10, damp=0.0, atol=0.0, btol=1e-3,
               callback=lambda xx: its.append(np.array(xx).copy()))
    np.savez_compressed(os.path.join(OUT, "solvers_precond.npz"), d=d, p=p.ravel(), z0=z0,
                        x=out[0], istop=out[1], iiter=out[2], r1=out[3], cost=out[10],
                        iterates=np.array(its))
    print("wrote solvers_precond")

    # 12) single traveltime table: mode='byot' with trav of shape (ni, ns*nr)
    # (kirchhoff.py:396-398, 684-725); a second table shifted so that some
    # times are negative (itrav truncates toward zero: -1 < t/dt < 0 -> 0)
    rng2 = np.random.default_rng(123)
    ts, tr, _, _, _, _ = Kirchhoff._traveltime_table(z, x, s2d, r2d, v0, mode="analytic")
    tt = (ts[:, :, None] + tr[:, None, :]).reshape(ts.shape[0], -1)
    tt = tt * (1.0 + 0.2 * np.cos(np.arange(tt.shape[0]) / 5.0))[:, None]
    for name, table in (("k2d_single", tt), ("k2d_single_neg", tt - 0.5 * tt.mean())):
        K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="byot", trav=table, engine="numpy")
        xin = rng2.standard_normal(K.ni)
        din = rng2.standard_normal(K.shape[0])
        spread = K._kirch_matvec(xin, np.zeros((K.nsnr, K.nt)), K.nsnr, K.nt, K.ni, K.itrav, K.travd)
        gather = K._kirch_rmatvec(din.reshape(K.nsnr, K.nt), np.zeros(K.ni), K.nsnr, K.nt, K.ni, K.itrav,
                                  K.travd)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), trav_table=table, m_in=xin, d_in=din,
                            fwd=np.asarray(K @ xin), adj=np.asarray(K.H @ din), spread=spread, gather=gather,
                            itrav=K.itrav, travd=K.travd, wav=np.asarray(K.wav), wavc=wavc, ns=K.ns, nr=K.nr,
                            nt=K.nt, ni=int(K.ni), dt=float(K.dt), nz=K.nz, dynamic=False, vel_scalar=v0,
                            **geom2d())
        print("wrote", name)

    # 13) preconditioned inversion (cls_leastsquares.py:768-1021): CGLS on Op @ P,
    # x = P p, on the dynamic operator of case 11 and on a dense matrix
    from pylops.basicoperators import MatrixMult
    from pylops.optimization.leastsquares import preconditioned_inversion

    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=True,
                  angleaperture=None, engine="numpy")
    refl = np.zeros((PAR["nx"], PAR["nz"]))
    refl[:, PAR["nz"] // 2] = 1
    refl[:, 3 * PAR["nz"] // 4] = 1
    d = K @ refl.ravel()
    p = 1.0 + 0.1 * np.tile(np.arange(PAR["nz"]), PAR["nx"])
    xk = preconditioned_inversion(K, d, Diagonal(p), engine="pylops", niter=8, tol=1e-10)
    rng3 = np.random.default_rng(7)
    A = rng3.standard_normal((40, 25))
    pa = rng3.uniform(0.5, 2.0, 25)
    ya = A @ rng3.standard_normal(25)
    xa_s = preconditioned_inversion(MatrixMult(A), ya, Diagonal(pa), engine="scipy", iter_lim=30)
    xa_p = preconditioned_inversion(MatrixMult(A), ya, Diagonal(pa), engine="pylops", niter=12, tol=1e-12)
    np.savez_compressed(os.path.join(OUT, "precond_inversion.npz"), d=d, p=p, xk=xk[0], xk_iit=xk[2],
                        xk_r1=xk[3], A=A, pa=pa, ya=ya, xa_scipy=xa_s[0], xa_scipy_iit=xa_s[2],
                        xa_pylops=xa_p[0], xa_pylops_iit=xa_p[2], xa_pylops_r1=xa_p[3])
    print("wrote precond_inversion")

    # 14) 2-D non-stationary convolution (signalprocessing/nonstatconvolve2d.py),
    # filters on a coarse grid that leaves image points outside it on every side
    from pylops.signalprocessing import NonStationaryConvolve2D

    rng4 = np.random.default_rng(11)
    nxc, nzc = 60, 80
    ihx = np.arange(5, 55, 12)
    ihz = np.arange(3, 77, 14)
    hsc = rng4.standard_normal((len(ihx), len(ihz), 9, 11))
    C = NonStationaryConvolve2D(dims=(nxc, nzc), hs=hsc, ihx=ihx, ihz=ihz, engine="numpy")
    xc = rng4.standard_normal((nxc, nzc))
    yc = rng4.standard_normal((nxc, nzc))
    np.savez_compressed(os.path.join(OUT, "nsconv2d.npz"), hs=hsc, ihx=ihx, ihz=ihz, x_in=xc, y_in=yc,
                        fwd=(C @ xc.ravel()).reshape(nxc, nzc), adj=(C.H @ yc.ravel()).reshape(nxc, nzc))
    print("wrote nsconv2d")


def wavfilter_cases():
    """15) wavfilter=True: the wavelet reshaped by sqrt(j omega) in 2-D and by
    -j omega in 3-D (kirchhoff.py:395-398, 659-681)."""
    rng = np.random.default_rng(2024)
    K = Kirchhoff(z, x, t, s2d, r2d, v0, wav, wavc, mode="analytic", dynamic=False, wavfilter=True,
                  engine="numpy")
    _save("k2d_wavfilter", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc, wavfilter_in=True, wav_in=wav), geometry=geom2d())
    s3d6 = s3d[:, ::4].copy()
    K = Kirchhoff(z, x, t, s3d6, r3d, v0, wav, wavc, y=y, mode="analytic", dynamic=True,
                  angleaperture=45.0, wavfilter=True, engine="numpy")
    _save("k3d_wavfilter", K, rng.standard_normal(K.ni), rng.standard_normal(K.shape[0]),
          extra=dict(vel_scalar=v0, wavc=wavc, angleaperture_in=45.0, wavfilter_in=True, wav_in=wav),
          geometry=dict(z=z, x=x, t=t, srcs=s3d6, recs=r3d, y=y))


CASES = {"all": main, "wavfilter": wavfilter_cases}

if __name__ == "__main__":
    # python make_golden.py [all|wavfilter ...]: the named groups (default all)
    for name in (sys.argv[1:] or ["all", "wavfilter"]):
        CASES[name]()
