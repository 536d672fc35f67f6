"""FP64 NumPy oracle for the Kirchhoff demigration/migration path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
The product (``pylops_gb300``) never imports or calls anything in ``oracle/``.

It restates, in vectorised float64 NumPy, the algorithm of PyLops'
``pylops.waveeqprocessing.Kirchhoff`` (PyLops 2.5.0) and of the pieces it
calls.  Each function cites the reference file:line it follows.  Loop order
over (source, receiver) and the per-image-point arithmetic follow the
reference's ``numpy``/``numba`` engine exactly, including its quirks:

* time index by truncation ``int(t/dt)`` and the validity test
  ``0 <= it < nt - 1`` (``kirchhoff.py:745-751``);
* angle-aperture taper index ``int(20 * (|a| - amin) // (amax - amin))``
  (``kirchhoff.py:845-864``);
* the offset-aperture taper index ``int(20 * ((ap - apmin) // dap))`` which is
  always 0 inside the aperture, so only the hard cut-off acts
  (``kirchhoff.py:869-880``);
* 3-D receiver angles signed with the *source* gradient
  (``kirchhoff.py:386-393``).

Pinned against golden vectors produced by the reference itself
(``tests/golden/make_golden.py``; checked by ``tests/test_oracle.py``).
"""

from __future__ import annotations

import numpy as np

__all__ = [
    "ricker",
    "aperture_taper",
    "identify_geometry",
    "traveltime_table_analytic",
    "traveltime_table_eikonal",
    "angles_from_gradients",
    "pad_wavelet",
    "conv_same",
    "kirch_matvec",
    "kirch_rmatvec",
    "KirchhoffOracle",
    "lsqr",
    "cgls",
]


# ----------------------------------------------------------------------------
# small utilities
# ----------------------------------------------------------------------------
def ricker(t, f0=10.0):
    """Ricker wavelet on a symmetric axis (``pylops/utils/wavelets.py:167-205``)."""
    t = np.asarray(t, dtype=np.float64)
    if len(t) % 2 == 0:  # _tcrop, wavelets.py
        t = t[:-1]
    t = np.concatenate((np.flipud(-t[1:]), t), axis=0)
    a = (np.pi * f0 * t) ** 2
    w = (1.0 - 2.0 * a) * np.exp(-a)
    wcenter = int(np.argmax(np.abs(w)))
    return w, t, wcenter


def aperture_taper():
    """21-sample tail of a 41-sample Hanning mask with 20-sample edges
    (``kirchhoff.py:412`` -> ``pylops/utils/tapers.py:18-57``)."""
    han = np.hanning(2 * 20 - 1)
    st = han[:20]
    full = np.concatenate([st, np.ones(41 - 40), np.flipud(st)])
    return full[20:]


def identify_geometry(z, x, srcs, recs, y=None):
    """``Kirchhoff._identify_geometry`` (``kirchhoff.py:457-500``)."""
    ns, nr = srcs.shape[1], recs.shape[1]
    nz, nx = len(z), len(x)
    dz = np.abs(z[1] - z[0])
    dx = np.abs(x[1] - x[0])
    if y is None:
        return dict(ndims=2, shiftdim=0, dims=np.array([nx, nz]), ny=1, nx=nx,
                    nz=nz, ns=ns, nr=nr, dy=None, dx=dx, dz=dz,
                    dsamp=np.array([dx, dz]), origin=np.array([x[0], z[0]]))
    ny = len(y)
    dy = np.abs(y[1] - y[0])
    return dict(ndims=3, shiftdim=1, dims=np.array([ny, nx, nz]), ny=ny, nx=nx,
                nz=nz, ns=ns, nr=nr, dy=dy, dx=dx, dz=dz,
                dsamp=np.array([dy, dx, dz]), origin=np.array([y[0], x[0], z[0]]))


def traveltime_table_analytic(z, x, srcs, recs, vel, y=None):
    """Analytic (constant velocity) tables, ``kirchhoff.py:576-607`` and the
    gradient step ``kirchhoff.py:642-648``.

    Returns trav_srcs (ni, ns), trav_recs (ni, nr), dist_srcs, dist_recs and the
    per-axis traveltime gradients (lists of arrays shaped ``(*dims, ns|nr)``).
    """
    g = identify_geometry(z, x, srcs, recs, y=y)
    if not isinstance(vel, (float, int)):
        raise ValueError("vel must be scalar for mode=analytical")
    if g["ndims"] == 2:
        X, Z = np.meshgrid(x, z, indexing="ij")
        X, Z = X.ravel(), Z.ravel()
        Y = None
    else:
        Y, X, Z = np.meshgrid(y, x, z, indexing="ij")
        Y, X, Z = Y.ravel(), X.ravel(), Z.ravel()
    sd = g["shiftdim"]

    def _d2(pts):
        out = np.zeros((X.size, pts.shape[1]))
        for i, p in enumerate(pts.T):
            out[:, i] = (X - p[0 + sd]) ** 2 + (Z - p[1 + sd]) ** 2
            if Y is not None:
                out[:, i] += (Y - p[0]) ** 2
        return out

    trav_srcs = np.sqrt(_d2(srcs)) / vel
    trav_recs = np.sqrt(_d2(recs)) / vel
    dist_srcs = trav_srcs * vel
    dist_recs = trav_recs * vel
    dims = g["dims"]
    axes = tuple(range(g["ndims"]))
    grad_s = np.gradient(trav_srcs.reshape(*dims, g["ns"]), *g["dsamp"], axis=axes)
    grad_r = np.gradient(trav_recs.reshape(*dims, g["nr"]), *g["dsamp"], axis=axes)
    return trav_srcs, trav_recs, dist_srcs, dist_recs, grad_s, grad_r


def traveltime_table_eikonal(z, x, srcs, recs, vel, y=None):
    """Eikonal tables, ``kirchhoff.py:609-638`` (one fast-marching solve per
    source and per receiver, for the traveltimes with ``vel`` and for the
    distances with unit speed; the point at ``round((p - origin)/dsamp)``)
    and the gradient step ``kirchhoff.py:642-648``.  The fast marching is
    the C restatement ``oracle/eikonal_oracle.c`` of the method scikit-fmm
    implements (scikit-fmm itself is not available).  Same returns as
    :func:`traveltime_table_analytic`."""
    from oracle.kirch_oracle_c import eikonal_tables

    g = identify_geometry(z, x, srcs, recs, y=y)
    dims = tuple(int(d) for d in g["dims"])
    vel = np.asarray(vel, dtype=np.float64).reshape(dims)
    origin, dsamp = g["origin"], g["dsamp"]

    def _points(p):
        return np.round((p.T - origin) / dsamp).astype(np.int32)

    trav_srcs, dist_srcs = eikonal_tables(dims, dsamp, vel, _points(srcs))
    trav_recs, dist_recs = eikonal_tables(dims, dsamp, vel, _points(recs))
    axes = tuple(range(g["ndims"]))
    grad_s = np.gradient(trav_srcs.reshape(*dims, g["ns"]), *dsamp, axis=axes)
    grad_r = np.gradient(trav_recs.reshape(*dims, g["nr"]), *dsamp, axis=axes)
    return trav_srcs, trav_recs, dist_srcs, dist_recs, grad_s, grad_r


def angles_from_gradients(grad_s, grad_r, ndims, ni, ns, nr):
    """Source/receiver angles with the vertical (``kirchhoff.py:364-393``).

    2-D: ``arctan2(dT/dx, dT/dz)``; 3-D: ``sign(dTs/dx) * arccos(dT/dz / |grad T|)``
    (the receiver angle also takes the *source* gradient's sign).
    """
    if ndims == 2:
        a_s = np.arctan2(grad_s[0], grad_s[1]).reshape(ni, ns)
        a_r = np.arctan2(grad_r[0], grad_r[1]).reshape(ni, nr)
    else:
        gs = np.concatenate([grad_s[i][np.newaxis] for i in range(3)])
        gr = np.concatenate([grad_r[i][np.newaxis] for i in range(3)])
        a_s = (np.sign(gs[1]) * np.arccos(gs[-1] / np.sqrt(np.sum(gs ** 2, axis=0)))).reshape(ni, ns)
        a_r = (np.sign(gs[1]) * np.arccos(gr[-1] / np.sqrt(np.sum(gr ** 2, axis=0)))).reshape(ni, nr)
    return a_s, a_r


def wavelet_reshaping(wav, dt, dimsrc, dimrec, ndims):
    """``wavfilter=True`` (``kirchhoff.py:659-681``): the wavelet's spectrum
    times sqrt(j 2 pi f) in 2-D and -j 2 pi f in 3-D (rfft / irfft of the
    wavelet's own length); a 2-D source or receiver in a 3-D model raises."""
    f = np.fft.rfftfreq(len(wav), dt)
    omega = 2 * np.pi * f
    if dimsrc == 2 and ndims == 2:
        mult = np.sqrt(1j * omega)
    elif ndims == 3 and (dimsrc == 2 or dimrec == 2):
        raise NotImplementedError("2.D wavelet currently not available")
    else:
        mult = -1j * omega
    return np.fft.irfft(np.fft.rfft(wav, n=len(wav)) * mult, n=len(wav))


def pad_wavelet(h, offset):
    """Zero-pad a filter the way ``_Convolve1Dshort`` does
    (``pylops/signalprocessing/convolve1d.py:76-88``) so that a plain
    ``'same'`` convolution centres it on sample ``offset``."""
    h = np.asarray(h, dtype=np.float64)
    nh = h.size
    if offset > nh - 1:
        raise ValueError("offset must be smaller than h.shape[axis] - 1")
    off = 2 * (nh // 2 - int(offset))
    if nh % 2 == 0:
        off -= 1
    if off != 0:
        h = np.pad(h, (max(off, 0), -min(off, 0)))
    return h


def conv_same(x2d, h):
    """``fftconvolve(x, h, mode='same', axes=1)`` restated as a direct FIR in
    float64 (``convolve1d.py:100-107``, ``backend.py:189``):
    ``y[n] = sum_k h[k] x[n + (L-1)//2 - k]`` with zero padding."""
    x2d = np.asarray(x2d, dtype=np.float64)
    L = h.size
    c = (L - 1) // 2
    nt = x2d.shape[1]
    y = np.zeros_like(x2d)
    for k in range(L):
        s = c - k  # y[n] += h[k] * x[n + s]
        if s >= 0:
            if s < nt:
                y[:, : nt - s] += h[k] * x2d[:, s:]
        else:
            if -s < nt:
                y[:, -s:] += h[k] * x2d[:, : nt + s]
    return y


# ----------------------------------------------------------------------------
# the two hot loops
# ----------------------------------------------------------------------------
def _tindex(trav, dt):
    # kirchhoff.py:742-745 (forward) and 772-774 (adjoint): truncation toward 0
    tt = trav / dt
    it = tt.astype(np.int64)  # numpy astype truncates toward zero, like int()
    return it, tt - it


def _dynamic_weight(isrc, irec, nr, dyn):
    """Per-image-point weight ``damp * aptap`` for one (src, rec) pair, or 0
    where the angle or offset aperture rejects it (``kirchhoff.py:820-880``)."""
    a_s = dyn["angle_srcs"][:, isrc]
    a_r = dyn["angle_recs"][:, irec]
    damp = 2.0 * np.cos((a_s - a_r) / 2.0) * dyn["amp_srcs"][:, isrc] * dyn["amp_recs"][:, irec] / dyn["vel"]
    amin, amax = dyn["angleaperture"]
    apmin, apmax = dyn["aperture"]
    tap = dyn["aperturetap"]
    dang = amax - amin
    dap = apmax - apmin
    abs_s, abs_r = np.abs(a_s), np.abs(a_r)
    ok = (abs_s < amax) & (abs_r < amax)
    aptap = np.ones_like(damp)
    with np.errstate(invalid="ignore", divide="ignore"):
        ms = ok & (abs_s >= amin)
        idx = np.zeros(abs_s.shape, dtype=np.int64)
        idx[ms] = (20 * (abs_s[ms] - amin) // dang).astype(np.int64)
        aptap[ms] *= tap[idx[ms]]
        mr = ok & (abs_r >= amin)
        idx = np.zeros(abs_r.shape, dtype=np.int64)
        idx[mr] = (20 * (abs_r[mr] - amin) // dang).astype(np.int64)
        aptap[mr] *= tap[idx[mr]]
    ni = a_s.size
    iz = np.arange(ni) % dyn["nz"]
    pair = isrc * nr + irec
    ap = np.abs(dyn["six"][pair] - dyn["rix"][pair]) / (iz + 1)
    okap = ok & (ap < apmax)
    mp = okap & (ap >= apmin)
    if np.any(mp):
        idx = (20 * ((ap[mp] - apmin) // dap)).astype(np.int64)
        aptap[mp] *= tap[idx]
    return np.where(okap, damp * aptap, 0.0)


def kirch_matvec(x, ns, nr, nt, ni, dt, trav_srcs, trav_recs, dyn=None):
    """Forward spreading, before the wavelet.

    Kinematic: ``Kirchhoff._travsrcrec_kirch_matvec`` (``kirchhoff.py:728-752``);
    dynamic: ``Kirchhoff._ampsrcrec_kirch_matvec`` (``kirchhoff.py:784-889``).
    Returns y of shape (ns*nr, nt) in float64.
    """
    x = np.asarray(x, dtype=np.float64).ravel()
    y = np.zeros((ns * nr, nt))
    for isrc in range(ns):
        for irec in range(nr):
            it, w = _tindex(trav_srcs[:, isrc] + trav_recs[:, irec], dt)
            v = x if dyn is None else x * _dynamic_weight(isrc, irec, nr, dyn)
            ok = (it >= 0) & (it < nt - 1)
            row = y[isrc * nr + irec]
            row += np.bincount(it[ok], weights=v[ok] * (1 - w[ok]), minlength=nt)[:nt]
            row += np.bincount(it[ok] + 1, weights=v[ok] * w[ok], minlength=nt)[:nt]
    return y


def kirch_rmatvec(d, ns, nr, nt, ni, dt, trav_srcs, trav_recs, dyn=None):
    """Adjoint gathering, after the wavelet correlation.

    Kinematic: ``Kirchhoff._travsrcrec_kirch_rmatvec`` (``kirchhoff.py:755-781``);
    dynamic: ``Kirchhoff._ampsrcrec_kirch_rmatvec`` (``kirchhoff.py:892-1001``).
    Returns the image of length ni in float64.
    """
    d = np.asarray(d, dtype=np.float64).reshape(ns * nr, nt)
    img = np.zeros(ni)
    for isrc in range(ns):
        for irec in range(nr):
            it, w = _tindex(trav_srcs[:, isrc] + trav_recs[:, irec], dt)
            ok = (it >= 0) & (it < nt - 1)
            row = d[isrc * nr + irec]
            itc = np.where(ok, it, 0)
            val = np.where(ok, row[itc] * (1 - w) + row[np.minimum(itc + 1, nt - 1)] * w, 0.0)
            if dyn is not None:
                val = val * _dynamic_weight(isrc, irec, nr, dyn)
            img += val
    return img


def single_table_index(trav, dt):
    """``itrav = (trav / dt).astype('int32')``, ``travd = trav / dt - itrav``
    (``kirchhoff.py:396-398``) for a single table of shape (ni, ns*nr)."""
    tt = np.asarray(trav, dtype=np.float64) / dt
    it = tt.astype(np.int32)
    return it, tt - it


def trav_matvec(x, nsnr, nt, ni, itrav, travd):
    """Single-table forward spreading, ``Kirchhoff._trav_kirch_matvec``
    (``kirchhoff.py:684-704``); y of shape (nsnr, nt)."""
    x = np.asarray(x, dtype=np.float64).ravel()
    y = np.zeros((nsnr, nt))
    for k in range(nsnr):
        it, w = itrav[:, k].astype(np.int64), travd[:, k]
        ok = (it >= 0) & (it < nt - 1)
        y[k] += np.bincount(it[ok], weights=x[ok] * (1 - w[ok]), minlength=nt)[:nt]
        y[k] += np.bincount(it[ok] + 1, weights=x[ok] * w[ok], minlength=nt)[:nt]
    return y


def trav_rmatvec(d, nsnr, nt, ni, itrav, travd):
    """Single-table adjoint gathering, ``Kirchhoff._trav_kirch_rmatvec``
    (``kirchhoff.py:707-725``); image of length ni."""
    d = np.asarray(d, dtype=np.float64).reshape(nsnr, nt)
    img = np.zeros(ni)
    for k in range(nsnr):
        it, w = itrav[:, k].astype(np.int64), travd[:, k]
        ok = (it >= 0) & (it < nt - 1)
        itc = np.where(ok, it, 0)
        img += np.where(ok, d[k, itc] * (1 - w) + d[k, np.minimum(itc + 1, nt - 1)] * w, 0.0)
    return img


# ----------------------------------------------------------------------------
# operator wrapper (constructor semantics of kirchhoff.py:234-455)
# ----------------------------------------------------------------------------
class KirchhoffOracle:
    """FP64 restatement of ``Kirchhoff(...)`` for ``mode in {'analytic','eikonal','byot'}``.

    ``trav``/``amp`` (byot) must be tuples of per-source and per-receiver
    tables, as for the reference's ``travsrcrec`` path.  ``vel`` is the scalar
    velocity (analytic) or the velocity model used for the dynamic weights.
    """

    def __init__(self, z, x, t, srcs, recs, vel, wav, wavcenter, y=None,
                 mode="analytic", dynamic=False, trav=None, amp=None,
                 aperture=None, angleaperture=90.0, wavfilter=False):
        g = identify_geometry(z, x, srcs, recs, y=y)
        self.g = g
        self.ndims, self.nx, self.nz, self.ny = g["ndims"], g["nx"], g["nz"], g["ny"]
        ns, nr = g["ns"], g["nr"]
        self.dt = t[1] - t[0]
        self.nt = len(t)
        self.dynamic = dynamic
        dims = g["dims"]
        ni = int(np.prod(dims))
        if dynamic:  # kirchhoff.py:287-301
            dx = x[1] - x[0]
            if self.ndims == 2:
                self.six = np.tile((srcs[0] - x[0]) // dx, (nr, 1)).T.astype(int).ravel()
                self.rix = np.tile((recs[0] - x[0]) // dx, (ns, 1)).astype(int).ravel()
            else:
                self.six = np.zeros(nr * ns)
                self.rix = np.zeros(nr * ns)
        if mode in ("analytic", "eikonal"):
            table = traveltime_table_analytic if mode == "analytic" else traveltime_table_eikonal
            ts, tr, ds, dr, gs, gr = table(z, x, srcs, recs, vel, y=y)
            self.trav_srcs, self.trav_recs = ts, tr
            if dynamic:  # kirchhoff.py:316-330
                maxdist = 1e-2 * (np.max(ds) + np.max(dr))
                if self.ndims == 2:
                    self.amp_srcs, self.amp_recs = 1.0 / np.sqrt(ds + maxdist), 1.0 / np.sqrt(dr + maxdist)
                else:
                    self.amp_srcs, self.amp_recs = 1.0 / (ds + maxdist), 1.0 / (dr + maxdist)
        elif mode == "byot":
            self.trav_srcs, self.trav_recs = trav
            if dynamic:  # kirchhoff.py:344-360 (gradients without spacing)
                self.amp_srcs, self.amp_recs = amp
                axes = np.arange(self.ndims)
                gs = np.gradient(self.trav_srcs.reshape(*dims, ns), axis=axes)
                gr = np.gradient(self.trav_recs.reshape(*dims, nr), axis=axes)
        else:
            raise NotImplementedError("method must be analytic, eikonal or byot")
        if dynamic:
            self.angle_srcs, self.angle_recs = angles_from_gradients(gs, gr, self.ndims, ni, ns, nr)
        # kirchhoff.py:395-398
        self.wav = wavelet_reshaping(wav, self.dt, srcs.shape[0], recs.shape[0], self.ndims) if wavfilter else wav
        self.h = pad_wavelet(self.wav, wavcenter)
        self.aperturetap = aperture_taper()
        if aperture is not None and self.ndims == 3:
            aperture = None
        ap = (self.nx + 1,) if aperture is None else np.atleast_1d(np.asarray(aperture, dtype=np.float64))
        self.aperture = np.array([0.8 * ap[0], ap[0]]) if len(ap) == 1 else np.asarray(ap, dtype=np.float64)
        angleaperture = [0.0, 1000.0] if angleaperture is None else angleaperture
        aa = np.deg2rad(np.atleast_1d(np.asarray(angleaperture, dtype=np.float64)))
        self.angleaperture = np.array([0.8 * aa[0], aa[0]]) if len(aa) == 1 else aa
        self.ns, self.nr, self.ni = ns, nr, ni
        if dynamic:
            self.vel = (np.asarray(vel, dtype=np.float64).flatten()
                        if not isinstance(vel, (float, int)) else vel * np.ones(ni))
        self.shape = (ns * nr * self.nt, ni)

    def _dyn(self):
        if not self.dynamic:
            return None
        return dict(vel=self.vel, amp_srcs=self.amp_srcs, amp_recs=self.amp_recs,
                    angle_srcs=self.angle_srcs, angle_recs=self.angle_recs,
                    aperture=self.aperture, angleaperture=self.angleaperture,
                    aperturetap=self.aperturetap, nz=self.nz, six=self.six, rix=self.rix)

    def spread(self, x):
        return kirch_matvec(x, self.ns, self.nr, self.nt, self.ni, self.dt,
                            self.trav_srcs, self.trav_recs, self._dyn())

    def gather(self, d):
        return kirch_rmatvec(d, self.ns, self.nr, self.nt, self.ni, self.dt,
                             self.trav_srcs, self.trav_recs, self._dyn())

    def matvec(self, x):
        """``Kirchhoff._matvec`` (``kirchhoff.py:1048-1094``): spread then wavelet."""
        return conv_same(self.spread(x), self.h).ravel()

    def rmatvec(self, d):
        """``Kirchhoff._rmatvec`` (``kirchhoff.py:1096-1143``): correlate then gather."""
        dc = conv_same(np.asarray(d, dtype=np.float64).reshape(self.ns * self.nr, self.nt), self.h[::-1].copy())
        return self.gather(dc)


# ----------------------------------------------------------------------------
# solvers (pylops/optimization/cls_basic.py), float64 host restatement
# ----------------------------------------------------------------------------
def cgls(matvec, rmatvec, y, nx, niter=10, damp=0.0, tol=1e-4, x0=None):
    """``CGLS`` setup/step/run (``cls_basic.py:432-608``), including the
    quirk that the x0 setup uses the unsquared ``damp`` (``:477``).
    Returns x, istop, iiter, r1norm, r2norm, cost, iterates."""
    y = np.asarray(y, dtype=np.float64)
    dampsq = damp ** 2
    if x0 is None:
        x = np.zeros(nx)
        s = y.copy()
        c = rmatvec(s)
    else:
        x = np.asarray(x0, dtype=np.float64).copy()
        s = y - matvec(x)
        c = rmatvec(s) - damp * x
    q = matvec(c)
    kold = abs(c @ c)
    cost = [float(np.linalg.norm(s))]
    cost1 = [float(np.sqrt(cost[0] ** 2 + damp * abs(x @ x)))]
    iiter = 0
    iterates = []
    while iiter < niter and kold > tol:
        a = kold / (q @ q + dampsq * (c @ c))
        x = x + a * c
        s = s - a * q
        r = rmatvec(s) - dampsq * x
        k = abs(r @ r)
        b = k / kold
        c = r + b * c
        q = matvec(c)
        kold = k
        iiter += 1
        cost.append(float(np.linalg.norm(s)))
        cost1.append(float(np.sqrt(cost[-1] ** 2 + dampsq * abs(x @ x))))
        iterates.append(x.copy())
    istop = 1 if kold < tol else 2
    return x, istop, iiter, kold, cost1[iiter], np.array(cost), iterates


def lsqr(matvec, rmatvec, y, nx, niter=10, damp=0.0, atol=1e-8, btol=1e-8,
         conlim=1e8, x0=None):
    """``LSQR`` setup/step (``cls_basic.py:835-1136``) in float64.
    Returns x, istop, iiter, r1norm, r2norm, anorm, acond, arnorm, xnorm,
    cost, iterates."""
    y = np.asarray(y, dtype=np.float64)
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    anorm = acond = ddnorm = res2 = xnorm = xxnorm = z = 0.0
    cs2, sn2 = -1.0, 0.0
    dampsq = damp ** 2
    if x0 is None:
        x = np.zeros(nx)
        u = y.copy()
    else:
        x = np.asarray(x0, dtype=np.float64).copy()
        u = y - matvec(x)
    alfa = 0.0
    beta = float(np.linalg.norm(u))
    if beta > 0:
        u = u / beta
        v = rmatvec(u)
        alfa = float(np.linalg.norm(v))
        if alfa > 0:
            v = v / alfa
    else:
        v = x.copy()
    w = v.copy()
    arnorm = arnorm0 = alfa * beta
    rhobar, phibar, bnorm = alfa, beta, beta
    rnorm = r1norm = r2norm = beta
    cost = [rnorm]
    iterates = []
    istop = 0
    iiter = 0
    while iiter < niter and istop == 0:
        u = matvec(v) - alfa * u
        beta = float(np.linalg.norm(u))
        if beta > 0:
            u = u / beta
            anorm = float(np.linalg.norm([anorm, alfa, beta, damp]))
            v = rmatvec(u) - beta * v
            alfa = float(np.linalg.norm(v))
            if alfa > 0:
                v = v / alfa
        rhobar1 = float(np.linalg.norm([rhobar, damp]))
        cs1 = rhobar / rhobar1
        sn1 = damp / rhobar1
        psi = sn1 * phibar
        phibar = cs1 * phibar
        rho = float(np.linalg.norm([rhobar1, beta]))
        cs = rhobar1 / rho
        sn = beta / rho
        theta = sn * alfa
        rhobar = -cs * alfa
        phi = cs * phibar
        phibar = sn * phibar
        tau = sn * phi
        t1 = phi / rho
        t2 = -theta / rho
        dk = w / rho
        x = x + t1 * w
        w = v + t2 * w
        ddnorm = ddnorm + float(np.linalg.norm(dk)) ** 2
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = np.sqrt(xxnorm + zbar ** 2)
        gamma = float(np.linalg.norm([gambar, theta]))
        cs2 = gambar / gamma
        sn2 = theta / gamma
        z = rhs / gamma
        xxnorm = xxnorm + z ** 2
        acond = anorm * np.sqrt(ddnorm)
        res1 = phibar ** 2
        res2 = res2 + psi ** 2
        rnorm = np.sqrt(res1 + res2)
        arnorm = alfa * abs(tau)
        r1sq = rnorm ** 2 - dampsq * xxnorm
        r1norm = np.sqrt(abs(r1sq))
        cost.append(float(r1norm))
        if r1sq < 0:
            r1norm = -r1norm
        r2norm = rnorm
        test1 = rnorm / bnorm
        test2 = arnorm / arnorm0
        test3 = 1.0 / acond
        tt1 = test1 / (1.0 + anorm * xnorm / bnorm)
        rtol = btol + atol * anorm * xnorm / bnorm
        if iiter >= niter:
            istop = 7
        if 1 + test3 <= 1:
            istop = 6
        if 1 + test2 <= 1:
            istop = 5
        if 1 + tt1 <= 1:
            istop = 4
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        iiter += 1
        iterates.append(x.copy())
    return (x, istop, iiter, r1norm, r2norm, anorm, acond, arnorm, xnorm,
            np.array(cost), iterates)
