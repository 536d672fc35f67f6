"""ctypes wrapper of the C restatements ``oracle/kirch_oracle.c`` (the
numba loop nests) and ``oracle/eikonal_oracle.c`` (the fast-marching tables).

TEST INFRASTRUCTURE ONLY (tests, smoke check, the CPU-baseline leg and the
reference arm of bench.py).  ``build()`` compiles both with gcc/OpenMP into
one library under ``oracle/_build/``.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "kirch_oracle.c"), os.path.join(HERE, "eikonal_oracle.c")]
OUT = os.path.join(HERE, "_build", "libkirch_oracle.so")
_lib = None


def build(force=False):
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(s) for s in SRCS):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c99", *SRCS, "-o", OUT + ".tmp", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


class _Op(ctypes.Structure):
    _fields_ = [("ns", ctypes.c_int), ("nr", ctypes.c_int), ("nt", ctypes.c_int), ("nz", ctypes.c_int),
                ("ni", ctypes.c_int64), ("dt", ctypes.c_double),
                ("ts", ctypes.c_void_p), ("tr", ctypes.c_void_p), ("dynamic", ctypes.c_int),
                ("as_", ctypes.c_void_p), ("ar", ctypes.c_void_p), ("ans", ctypes.c_void_p),
                ("anr", ctypes.c_void_p), ("vel", ctypes.c_void_p),
                ("apmin", ctypes.c_double), ("apmax", ctypes.c_double), ("amin", ctypes.c_double),
                ("amax", ctypes.c_double), ("taper", ctypes.c_void_p), ("six", ctypes.c_void_p),
                ("rix", ctypes.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P = ctypes.c_void_p
        L.ko_spread.argtypes = [ctypes.POINTER(_Op), P, P, ctypes.c_int, ctypes.c_int]
        L.ko_gather.argtypes = [ctypes.POINTER(_Op), P, P, ctypes.c_int, ctypes.c_int]
        L.ko_conv.argtypes = [P, P, ctypes.c_int64, ctypes.c_int, P, ctypes.c_int]
        L.eo_tables.argtypes = [ctypes.c_int, P, P, P, ctypes.c_int, P, P, P, ctypes.c_int]
        L.eo_tables.restype = ctypes.c_int
        _lib = L
    return _lib


class COracle:
    """Float64 multi-threaded restatement of the reference's numba engine.

    Built from an object exposing the reference attributes (the GB300
    Kirchhoff or ``kirchhoff_oracle.KirchhoffOracle``) plus the padded filter.
    """

    def __init__(self, K, h_padded):
        c = lambda a, dt=np.float64: np.ascontiguousarray(np.asarray(a), dtype=dt)  # noqa: E731
        self.keep = [c(K.trav_srcs), c(K.trav_recs)]
        self.h = c(h_padded)
        op = _Op()
        op.ns, op.nr, op.nt, op.nz, op.ni, op.dt = K.ns, K.nr, K.nt, K.nz, int(K.ni), float(K.dt)
        op.ts, op.tr = self.keep[0].ctypes.data, self.keep[1].ctypes.data
        op.dynamic = int(bool(K.dynamic))
        if K.dynamic:
            arrs = [c(K.amp_srcs), c(K.amp_recs), c(K.angle_srcs), c(K.angle_recs), c(K.vel),
                    c(K.aperturetap), c(K.six, np.int64), c(K.rix, np.int64)]
            self.keep += arrs
            op.as_, op.ar, op.ans, op.anr, op.vel, op.taper, op.six, op.rix = [a.ctypes.data for a in arrs]
            op.apmin, op.apmax = float(K.aperture[0]), float(K.aperture[1])
            op.amin, op.amax = float(K.angleaperture[0]), float(K.angleaperture[1])
        self.op = op
        self.ns, self.nr, self.nt, self.ni = K.ns, K.nr, K.nt, int(K.ni)

    def spread(self, x, s0=0, s1=None):
        s1 = self.ns if s1 is None else s1
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros((self.ns * self.nr, self.nt))
        lib().ko_spread(ctypes.byref(self.op), x.ctypes.data, y.ctypes.data, s0, s1)
        return y

    def gather(self, d, s0=0, s1=None):
        s1 = self.ns if s1 is None else s1
        d = np.ascontiguousarray(d, dtype=np.float64).reshape(self.ns * self.nr, self.nt)
        img = np.zeros(self.ni)
        lib().ko_gather(ctypes.byref(self.op), d.ctypes.data, img.ctypes.data, s0, s1)
        return img

    def conv(self, x, adjoint=False):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.nt)
        y = np.empty_like(x)
        h = np.ascontiguousarray(self.h[::-1]) if adjoint else self.h
        lib().ko_conv(x.ctypes.data, y.ctypes.data, x.shape[0], self.nt, h.ctypes.data, h.size)
        return y

    def matvec(self, x):
        return self.conv(self.spread(x)).ravel()

    def rmatvec(self, d):
        return self.gather(self.conv(d, adjoint=True))


def eikonal_tables(dims, dsamp, speed, points, order=2, with_trav=True, with_dist=True):
    """Fast-marching tables of ``points`` (npts, nd) grid coordinates on a grid
    of shape ``dims`` with spacings ``dsamp``: (trav, dist), each (N, npts)
    or None, trav with the velocity ``speed`` (shape ``dims``), dist with
    speed 1."""
    dims = np.ascontiguousarray(dims, dtype=np.int32)
    nd = dims.size
    N = int(np.prod(dims))
    h = np.ascontiguousarray(dsamp, dtype=np.float64)
    pts = np.ascontiguousarray(points, dtype=np.int32).reshape(-1, nd)
    sp = np.ascontiguousarray(np.broadcast_to(np.asarray(speed, np.float64), tuple(dims)))
    trav = np.empty((N, pts.shape[0])) if with_trav else None
    dist = np.empty((N, pts.shape[0])) if with_dist else None
    rc = lib().eo_tables(nd, dims.ctypes.data, h.ctypes.data, sp.ctypes.data, pts.shape[0], pts.ctypes.data,
                         trav.ctypes.data if trav is not None else None,
                         dist.ctypes.data if dist is not None else None, order)
    if rc != 0:
        raise ValueError("eikonal oracle: bad arguments")
    return trav, dist
