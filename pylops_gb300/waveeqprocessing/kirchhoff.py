"""Kirchhoff demigration/migration operator on GB300.

Drop-in for ``pylops.waveeqprocessing.Kirchhoff`` (PyLops 2.5.0,
``pylops/waveeqprocessing/kirchhoff.py:40-1143``): same constructor,
attributes and ``LinearOperator`` behaviour.  Tables are built on the host
exactly as the reference builds them (analytic formulas, the package's own
fast-marching eikonal solver in place of scikit-fmm, or user tables), then
stored in HBM once; every ``matvec``/``rmatvec`` runs the sm_103a kernels of
``libpylops_gb300.so`` through its C ABI.  There is no host compute path:
all three ``engine`` names select the CUDA kernels.

Reassigning a table attribute (``Dop.trav_srcs = ...``, as the reference's
tests do) re-uploads the device copy before the next application.
"""

from __future__ import annotations

import ctypes
import logging
import warnings
from typing import Optional, Tuple, Union

import numpy as np

from .. import _native
from ..linearoperator import LinearOperator
from ..utils.backend import is_torch
from ..utils.tapers import taper

__all__ = ["Kirchhoff"]

logger = logging.getLogger(__name__)

_TABLE_ATTRS = ("trav", "trav_srcs", "trav_recs", "amp_srcs", "amp_recs", "angle_srcs", "angle_recs",
                "vel", "aperture", "angleaperture", "aperturetap", "six", "rix")
# tables built on the device, read back on first access (kgb_kirchhoff_get_table)
_DEVICE_TABLES = {"trav_srcs": 0, "trav_recs": 1, "amp_srcs": 2, "amp_recs": 3, "angle_srcs": 4, "angle_recs": 5}


def _value_or_sized_to_array(v, repeat: int = 1):
    try:
        len(v)
        return np.asarray(v)
    except TypeError:
        return np.array([v] * repeat)


class _WaveletOperator(LinearOperator):
    """The operator's wavelet convolution along time (``Kirchhoff.cop``):
    ``Convolve1D((ns*nr, nt), h=wav, offset=wavcenter, axis=1)``
    (``pylops/signalprocessing/convolve1d.py:57-116``) on the device."""

    def __init__(self, parent: "Kirchhoff", h, offset, dtype):
        super().__init__(dtype=np.dtype(dtype), dims=(parent.nsnr, parent.nt),
                         dimsd=(parent.nsnr, parent.nt), name="C")
        self._parent = parent
        self.h = h
        self.offset = offset

    def _apply(self, x, adjoint):
        p = self._parent
        p._sync_tables()
        L = _native.lib()
        if is_torch(x):
            import torch

            xx = x.to(device="cuda", dtype=torch.float32).contiguous()
            y = torch.empty_like(xx)
            _native.check(L.kgb_kirchhoff_wavelet(p._h, xx.data_ptr(), y.data_ptr(), int(adjoint),
                                                  torch.cuda.current_stream().cuda_stream))
            return y.to(getattr(torch, str(self.dtype)))
        import torch  # device staging for host vectors

        xx = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device="cuda")
        y = torch.empty_like(xx)
        _native.check(L.kgb_kirchhoff_wavelet(p._h, xx.data_ptr(), y.data_ptr(), int(adjoint),
                                              torch.cuda.current_stream().cuda_stream))
        return y.cpu().numpy().astype(self.dtype, copy=False)

    def _matvec(self, x):
        return self._apply(x, False)

    def _rmatvec(self, x):
        return self._apply(x, True)


_PINNED_MAX_BYTES = 1 << 31


def _pinned_empty(n: int) -> np.ndarray:
    """A float32 host array in page-locked memory from torch's caching host
    allocator: the device-to-host copy of a result runs at full speed and,
    once the caller drops the array, the block is reused by the next call
    instead of faulting in fresh pages.  Page-locked memory is a limited
    host resource that the allocator keeps once used, so results above 2 GiB
    are ordinary (pageable) arrays."""
    if 4 * n > _PINNED_MAX_BYTES:
        return np.empty(n, dtype=np.float32)
    import torch

    return torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()


class Kirchhoff(LinearOperator):
    r"""Kirchhoff demigration operator (``kirchhoff.py:40-256``).

    Parameters are those of the reference: ``z, x, t, srcs, recs, vel, wav,
    wavcenter, y=None, mode='eikonal', wavfilter=False, dynamic=False,
    trav=None, amp=None, aperture=None, angleaperture=90., snell=None,
    engine='numpy', dtype='float64', name='K'``.

    Computation is float32 with float32 accumulation on the device whatever
    ``dtype`` is; ``dtype`` sets the type of returned host arrays.
    """

    def __init__(
        self,
        z,
        x,
        t,
        srcs,
        recs,
        vel,
        wav,
        wavcenter: int,
        y=None,
        mode: str = "eikonal",
        wavfilter: bool = False,
        dynamic: bool = False,
        trav=None,
        amp=None,
        aperture=None,
        angleaperture: Union[float, Tuple[float, float]] = 90.0,
        snell=None,
        engine: str = "numpy",
        dtype="float64",
        name: str = "K",
        tables: str = "device",
    ) -> None:
        if engine not in ["numpy", "numba", "cuda"]:
            raise KeyError("engine must be numpy or numba or cuda")
        if tables not in ("device", "host"):
            raise ValueError("tables must be 'device' or 'host'")
        object.__setattr__(self, "_h", None)
        object.__setattr__(self, "_dirty", set())
        object.__setattr__(self, "_device_built", False)
        (self.ndims, _, dims, self.ny, self.nx, self.nz, ns, nr, _, _, _, dsamp,
         origin) = Kirchhoff._identify_geometry(z, x, srcs, recs, y=y)
        self.dt = t[1] - t[0]
        self.nt = len(t)

        # per-trace source/receiver x indices for the offset aperture (kirchhoff.py:287-301)
        self.dynamic = dynamic
        if self.dynamic:
            dx = x[1] - x[0]
            if self.ndims == 2:
                self.six = np.tile((srcs[0] - x[0]) // dx, (nr, 1)).T.astype(int).ravel()
                self.rix = np.tile((recs[0] - x[0]) // dx, (ns, 1)).astype(int).ravel()
            else:
                self.six = np.zeros(nr * ns)
                self.rix = np.zeros(nr * ns)

        # tables (kirchhoff.py:303-362)
        self.travsrcrec = True
        # analytic and eikonal tables are built on the device (after the
        # operator exists, below)
        device_tables = tables == "device" and mode in ("analytic", "eikonal")
        if device_tables and mode == "analytic" and not isinstance(vel, (float, int)):
            raise ValueError("vel must be scalar for mode=analytical")
        if mode in ["analytic", "eikonal", "byot"]:
            if mode in ["analytic", "eikonal"] and device_tables:
                pass
            elif mode in ["analytic", "eikonal"]:
                (trav_srcs, trav_recs, dist_srcs, dist_recs, trav_srcs_grad,
                 trav_recs_grad) = Kirchhoff._traveltime_table(z, x, srcs, recs, vel, y=y, mode=mode)
                self.trav_srcs, self.trav_recs = trav_srcs, trav_recs
                if self.dynamic:
                    epsdist = 1e-2
                    self.maxdist = epsdist * (np.max(dist_srcs) + np.max(dist_recs))
                    if self.ndims == 2:
                        self.amp_srcs = 1.0 / np.sqrt(dist_srcs + self.maxdist)
                        self.amp_recs = 1.0 / np.sqrt(dist_recs + self.maxdist)
                    else:
                        self.amp_srcs = 1.0 / (dist_srcs + self.maxdist)
                        self.amp_recs = 1.0 / (dist_recs + self.maxdist)
            else:
                if isinstance(trav, tuple):
                    self.trav_srcs, self.trav_recs = trav
                else:
                    self.travsrcrec = False
                    self.trav = trav
                if self.dynamic and not self.travsrcrec:
                    raise NotImplementedError(
                        "separate traveltime tables must be provided when selecting mode=dynamic")
                if self.dynamic:
                    if isinstance(amp, tuple):
                        self.amp_srcs, self.amp_recs = amp
                    else:
                        raise NotImplementedError("separate amplitude tables must be provided ")
                    if self.travsrcrec:
                        # gradients without spacing, as the reference does (kirchhoff.py:353-360)
                        trav_srcs_grad = np.gradient(np.asarray(self.trav_srcs).reshape(*dims, ns),
                                                     axis=np.arange(self.ndims))
                        trav_recs_grad = np.gradient(np.asarray(self.trav_recs).reshape(*dims, nr),
                                                     axis=np.arange(self.ndims))
        else:
            raise NotImplementedError("method must be analytic, eikonal or byot")

        # angles with the vertical (kirchhoff.py:364-393)
        if self.dynamic and not device_tables:
            ni_ = int(np.prod(dims))
            if self.ndims == 2:
                self.angle_srcs = np.arctan2(trav_srcs_grad[0], trav_srcs_grad[1]).reshape(ni_, ns)
                self.angle_recs = np.arctan2(trav_recs_grad[0], trav_recs_grad[1]).reshape(ni_, nr)
            else:
                gs = np.concatenate([trav_srcs_grad[i][np.newaxis] for i in range(3)])
                gr = np.concatenate([trav_recs_grad[i][np.newaxis] for i in range(3)])
                self.angle_srcs = (np.sign(gs[1]) * np.arccos(gs[-1] / np.sqrt(np.sum(gs ** 2, axis=0)))
                                   ).reshape(ni_, ns)
                # The reference signs the receiver angle with the *source*
                # x-gradient, which only broadcasts when ns == nr; for ns != nr
                # (where the reference raises) the receiver's own gradient is used.
                sgn = np.sign(gs[1]) if ns == nr else np.sign(gr[1])
                self.angle_recs = (sgn * np.arccos(gr[-1] / np.sqrt(np.sum(gr ** 2, axis=0)))
                                   ).reshape(ni_, nr)

        # wavelet (kirchhoff.py:395-409)
        if wavfilter:
            self.wav = self._wavelet_reshaping(wav, self.dt, srcs.shape[0], recs.shape[0], self.ndims)
        else:
            self.wav = wav
        self.wavcenter = int(wavcenter)

        # apertures (kirchhoff.py:411-439)
        self.aperturetap = taper(41, 20, "hanning")[20:]
        if aperture is not None and self.ndims == 3:
            aperture = None
            warnings.warn("Aperture is forced to None as currently not implemented in 3D")
        if aperture is not None:
            warnings.warn("Aperture is currently defined as ratio of offset over depth, "
                          "and may be not ideal for highly heterogeneous media")
        ap = (self.nx + 1,) if aperture is None else _value_or_sized_to_array(aperture)
        if len(ap) == 1:
            ap = np.array([0.8 * ap[0], ap[0]])
        self.aperture = np.asarray(ap, dtype=np.float64)
        angleaperture = [0.0, 1000.0] if angleaperture is None else angleaperture
        aa = np.deg2rad(_value_or_sized_to_array(angleaperture))
        if len(aa) == 1:
            aa = np.array([0.8 * aa[0], aa[0]])
        self.angleaperture = np.asarray(aa, dtype=np.float64)

        # dimensions (kirchhoff.py:441-454)
        self.ns, self.nr = ns, nr
        self.nsnr = ns * nr
        self.ni = int(np.prod(dims))
        dims = tuple(dims) if self.ndims == 2 else (dims[0] * dims[1], dims[2])
        dimsd = (ns, nr, self.nt)
        super().__init__(dtype=np.dtype(dtype), dims=dims, dimsd=dimsd, name=name)
        if self.dynamic:
            self.vel = (np.asarray(vel).flatten() if not isinstance(vel, (float, int))
                        else vel * np.ones(int(np.prod(dims))))
        self.cop = _WaveletOperator(self, np.asarray(self.wav), self.wavcenter, dtype)
        if device_tables:
            self._create_native(build=dict(mode=mode, y=y, x=x, z=z, srcs=srcs, recs=recs, vel=vel))
        else:
            self._create_native()

    # single-table traveltimes: index and fraction (kirchhoff.py:395-398),
    # computed on first access (the device copy is made from `trav` itself,
    # with the same truncation)
    @property
    def itrav(self):
        if getattr(self, "travsrcrec", True):
            raise AttributeError("itrav exists for a single traveltime table only")
        return (np.asarray(self.trav) / self.dt).astype("int32")

    @property
    def travd(self):
        if getattr(self, "travsrcrec", True):
            raise AttributeError("travd exists for a single traveltime table only")
        return np.asarray(self.trav) / self.dt - self.itrav

    # ---------------------------------------------------------------- native
    def __setattr__(self, name, value):
        object.__setattr__(self, name, value)
        if name in _TABLE_ATTRS:
            self._dirty.add(name)

    def _create_native(self, build=None):
        L = _native.lib()
        wav = np.ascontiguousarray(np.asarray(self.wav, dtype=np.float64))
        h = ctypes.c_void_p()
        _native.check(L.kgb_kirchhoff_create(ctypes.byref(h), self.ns, self.nr, self.nt, self.ni, self.nz,
                                             float(self.dt), int(bool(self.dynamic)), _native.dptr(wav),
                                             int(wav.size), self.wavcenter))
        object.__setattr__(self, "_h", h)
        if build is None:
            self._dirty.update(_TABLE_ATTRS)
            self._sync_tables()
            return
        # tables on the device: traveltimes, distances, gradients, angles and
        # amplitudes computed where the kernels read them
        f64 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64))  # noqa: E731
        ax = [None if build["y"] is None else f64(build["y"]), f64(build["x"]), f64(build["z"])]
        vel = build["vel"]
        velv = f64([vel]) if isinstance(vel, (float, int)) else f64(vel).ravel()
        md = ctypes.c_double(0.0)
        if self.dynamic:
            dyn = [f64(self.aperture), f64(self.angleaperture), f64(self.aperturetap)]
            six = np.ascontiguousarray(np.asarray(self.six).astype(np.int64))
            rix = np.ascontiguousarray(np.asarray(self.rix).astype(np.int64))
            dptrs = [_native.dptr(a) for a in dyn] + [_native.i64ptr(six), _native.i64ptr(rix)]
        else:
            dptrs = [None] * 5
        _native.check(L.kgb_kirchhoff_build_tables(
            h, 0 if build["mode"] == "analytic" else 1, self.ndims,
            None if ax[0] is None else _native.dptr(ax[0]), 0 if ax[0] is None else ax[0].size,
            _native.dptr(ax[1]), ax[1].size, _native.dptr(ax[2]), ax[2].size,
            _native.dptr(f64(build["srcs"])), _native.dptr(f64(build["recs"])), _native.dptr(velv), velv.size,
            *dptrs, ctypes.byref(md)))
        if self.dynamic:
            object.__setattr__(self, "maxdist", md.value)
        object.__setattr__(self, "_device_built", True)
        self._dirty.clear()

    def __getattr__(self, name):
        # tables built on the device are read back on first access
        if name in _DEVICE_TABLES and self.__dict__.get("_device_built") and self.__dict__.get("_h") is not None:
            if name[:3] in ("amp", "ang") and not self.__dict__.get("dynamic"):
                raise AttributeError(name)
            n = self.__dict__["ns"] if name.endswith("srcs") else self.__dict__["nr"]
            out = np.empty((self.__dict__["ni"], n), dtype=np.float64)
            _native.check(_native.lib().kgb_kirchhoff_get_table(self.__dict__["_h"], _DEVICE_TABLES[name],
                                                                _native.dptr(out)))
            object.__setattr__(self, name, out)
            return out
        raise AttributeError(f"{type(self).__name__!r} object has no attribute {name!r}")

    def _sync_tables(self):
        if not self._dirty:
            return
        L = _native.lib()
        f64 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64))  # noqa: E731
        if not getattr(self, "travsrcrec", True):
            if "trav" in self._dirty:
                tt = f64(self.trav)
                if tt.size != self.ni * self.nsnr:
                    raise ValueError("traveltime table must be (ni, ns*nr)")
                _native.check(L.kgb_kirchhoff_set_traveltime_table(self._h, _native.dptr(tt)))
        elif {"trav_srcs", "trav_recs"} & self._dirty:
            ts, tr = f64(self.trav_srcs), f64(self.trav_recs)
            if ts.size != self.ni * self.ns or tr.size != self.ni * self.nr:
                raise ValueError("traveltime tables must be (ni, ns) and (ni, nr)")
            _native.check(L.kgb_kirchhoff_set_traveltimes(self._h, _native.dptr(ts), _native.dptr(tr)))
        if self.dynamic and ({"amp_srcs", "amp_recs", "angle_srcs", "angle_recs", "vel", "aperture",
                              "angleaperture", "aperturetap", "six", "rix"} & self._dirty):
            arrs = [f64(self.amp_srcs), f64(self.amp_recs), f64(self.angle_srcs), f64(self.angle_recs),
                    f64(self.vel), f64(self.aperture), f64(self.angleaperture), f64(self.aperturetap)]
            six = np.ascontiguousarray(np.asarray(self.six).astype(np.int64))
            rix = np.ascontiguousarray(np.asarray(self.rix).astype(np.int64))
            _native.check(L.kgb_kirchhoff_set_dynamic(self._h, *[_native.dptr(a) for a in arrs],
                                                      _native.i64ptr(six), _native.i64ptr(rix)))
        self._dirty.clear()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _native._lib is not None:
            try:
                _native._lib.kgb_kirchhoff_destroy(h)
            except Exception:  # pragma: no cover - interpreter shutdown
                pass
            object.__setattr__(self, "_h", None)

    @property
    def native_handle(self):
        """The ``kgb_kirchhoff*`` handle (tables synchronised)."""
        self._sync_tables()
        return self._h

    def info(self) -> dict:
        """Device-side layout and launch facts of this operator."""
        self._sync_tables()
        v = (ctypes.c_int64 * 16)()
        _native.check(_native.lib().kgb_kirchhoff_info(self._h, v))
        keys = ("ns", "nr", "nt", "ni", "frac_bits", "wavelet_len", "offset_gate", "dynamic", "nonneg",
                "adjoint_splits", "kernels_forward", "kernels_adjoint", "spread_variant", "spread_split",
                "max_bin_count")
        out = {k: int(v[i]) for i, k in enumerate(keys)}
        out["adjoint_variant"] = int(v[15]) & 3  # adjoint kernel in use (set_adjoint_variant)
        out["wait_error"] = int(v[15]) >> 2      # nonzero: a bounded wait of a kernel gave up
        return out

    def set_spread_variant(self, variant: int) -> None:
        """Select the forward kernel: 0 fixed-point atomics, 1 warp-binned
        (one trace per warp), 2 warp-binned (two traces per warp)."""
        _native.check(_native.lib().kgb_kirchhoff_set_variant(self._h, int(variant)))

    def set_adjoint_variant(self, variant: int) -> None:
        """Adjoint kernel of dynamic operators: 0 loads each source record in
        the gather (default), 1 keeps the next active source's record in
        flight (at most 64 sources), 2 stages the records by TMA; the image is
        the same bit for bit."""
        _native.check(_native.lib().kgb_kirchhoff_set_adjoint_variant(self._h, int(variant)))

    def set_weight_precision(self, precision: str = "float32") -> None:
        """Store the dynamic weights as ``'bfloat16'`` (8-byte table records,
        about 1e-3 relative change of the results) or ``'float32'``
        (default; 16-byte records, the mode that matches the reference to
        1e-5).  Traveltimes are exact in both."""
        if precision not in ("float32", "bfloat16"):
            raise ValueError("precision must be 'float32' or 'bfloat16'")
        self._sync_tables()
        _native.check(_native.lib().kgb_kirchhoff_set_weight_precision(self._h, int(precision == "bfloat16")))

    def autotune(self, variants=(0, 1, 2, 3), adjoint_variants=(0, 1, 2), reps: int = 3) -> dict:
        """Time the forward for each spread variant and, for dynamic
        operators, the adjoint for each adjoint variant on this operator's
        tables (random vectors, CUDA events on the current stream), keep the
        fastest of each and return {variant: ms} ({"adjoint v": ms} for the
        adjoint).  The spread variants give the same result to float32
        rounding (0 and 3 bit for bit), the adjoint variants bit for bit;
        which is fastest depends on the geometry."""
        import torch

        self._sync_tables()
        g = torch.Generator(device="cuda").manual_seed(0)
        m = torch.randn(self.ni, device="cuda", generator=g)
        d = torch.empty(self.shape[0], device="cuda")

        def timed(fn):
            fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            e1.synchronize()
            return e0.elapsed_time(e1) / reps

        times = {}
        for v in variants:
            self.set_spread_variant(v)
            times[v] = timed(lambda: self.apply_into(m, d))
        self.set_spread_variant(min(times, key=times.get))
        if self.dynamic and adjoint_variants:
            dd = torch.randn(self.shape[0], device="cuda", generator=g)
            adj = {}
            for v in adjoint_variants:
                self.set_adjoint_variant(v)
                adj[v] = timed(lambda: self.apply_into(dd, m, adjoint=True))
            self.set_adjoint_variant(min(adj, key=adj.get))
            times.update({f"adjoint {v}": t for v, t in adj.items()})
        return times

    @property
    def frac_bits(self) -> int:
        return self.info()["frac_bits"]

    # ---------------------------------------------------------------- apply
    def _run(self, x, which):
        """Apply forward (``which='forward'``/``'spread'``) or adjoint
        (``'adjoint'``/``'gather'``) on a numpy array (host copies inside the
        call) or a torch CUDA tensor (on torch's current stream)."""
        self._sync_tables()
        L = _native.lib()
        out_n = self.nsnr * self.nt if which in ("forward", "spread") else self.ni
        if is_torch(x):
            import torch

            xx = x.to(device="cuda", dtype=torch.float32).contiguous()
            y = torch.empty(out_n, dtype=torch.float32, device=xx.device)
            if which == "spread":
                y.zero_()
            fn = getattr(L, "kgb_kirchhoff_" + which)
            _native.check(fn(self._h, xx.data_ptr(), y.data_ptr(), torch.cuda.current_stream().cuda_stream))
            tdt = getattr(torch, str(self.dtype)) if str(self.dtype) in ("float32", "float64") else torch.float32
            return y if tdt == torch.float32 else y.to(tdt)
        xx = np.ascontiguousarray(np.asarray(x), dtype=np.float32)
        y = _pinned_empty(out_n)
        if which in ("forward", "adjoint"):
            fn = getattr(L, "kgb_kirchhoff_" + which + "_host")
            _native.check(fn(self._h, xx.ctypes.data, y.ctypes.data))
        else:
            import torch

            xd = torch.as_tensor(xx, device="cuda")
            yd = torch.zeros(out_n, dtype=torch.float32, device="cuda")
            fn = getattr(L, "kgb_kirchhoff_" + which)
            _native.check(fn(self._h, xd.data_ptr(), yd.data_ptr(), torch.cuda.current_stream().cuda_stream))
            y = yd.cpu().numpy()
        return y.astype(self.dtype, copy=False)

    def apply_into(self, x, out, adjoint: bool = False) -> None:
        """Forward (or adjoint) of a contiguous float32 CUDA tensor into the
        preallocated float32 CUDA tensor ``out``, on torch's current stream,
        without allocating."""
        import torch

        if not (is_torch(x) and is_torch(out)) or x.dtype != torch.float32 or out.dtype != torch.float32 \
                or not (x.is_cuda and out.is_cuda and x.is_contiguous() and out.is_contiguous()):
            raise TypeError("apply_into takes contiguous float32 CUDA tensors")
        n_in, n_out = (self.shape[0], self.shape[1]) if adjoint else (self.shape[1], self.shape[0])
        if x.numel() != n_in or out.numel() != n_out:
            raise ValueError(f"apply_into: sizes {x.numel()} -> {out.numel()}, expected {n_in} -> {n_out}")
        self._sync_tables()
        fn = _native.lib().kgb_kirchhoff_adjoint if adjoint else _native.lib().kgb_kirchhoff_forward
        _native.check(fn(self._h, x.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream))

    def _matvec(self, x):
        """Forward (``kirchhoff.py:1048-1094``)."""
        return self._run(x, "forward")

    def _rmatvec(self, x):
        """Adjoint (``kirchhoff.py:1096-1143``)."""
        return self._run(x, "adjoint")

    def spread(self, x):
        """Spreading without the wavelet (the reference's ``_kirch_matvec``)."""
        return self._run(x, "spread")

    def gather(self, x):
        """Gathering without the wavelet correlation (``_kirch_rmatvec``)."""
        return self._run(x, "gather")

    # ---------------------------------------------------------------- setup helpers
    @staticmethod
    def _identify_geometry(z, x, srcs, recs, y=None):
        """``Kirchhoff._identify_geometry`` (``kirchhoff.py:457-500``)."""
        ns, nr = srcs.shape[1], recs.shape[1]
        nz, nx = len(z), len(x)
        dz = np.abs(z[1] - z[0])
        dx = np.abs(x[1] - x[0])
        if y is None:
            return (2, 0, np.array([nx, nz]), 1, nx, nz, ns, nr, None, dx, dz, np.array([dx, dz]),
                    np.array([x[0], z[0]]))
        ny = len(y)
        dy = np.abs(y[1] - y[0])
        return (3, 1, np.array([ny, nx, nz]), ny, nx, nz, ns, nr, dy, dx, dz, np.array([dy, dx, dz]),
                np.array([y[0], x[0], z[0]]))

    @staticmethod
    def _traveltime_table(z, x, srcs, recs, vel, y=None, mode="eikonal"):
        """Traveltime, distance and gradient tables (``kirchhoff.py:503-657``).

        ``mode='analytic'`` uses the straight-ray formulas; ``mode='eikonal'``
        runs the package's fast-marching solver (``kgb_eikonal_tables``) with
        scikit-fmm's point-source convention.
        """
        (ndims, shiftdim, dims, ny, nx, nz, ns, nr, _, _, _, dsamp,
         origin) = Kirchhoff._identify_geometry(z, x, srcs, recs, y=y)
        if mode == "analytic":
            if not isinstance(vel, (float, int)):
                raise ValueError("vel must be scalar for mode=analytical")
            if ndims == 2:
                X, Z = np.meshgrid(x, z, indexing="ij")
                X, Z = X.ravel(), Z.ravel()
            else:
                Y, X, Z = np.meshgrid(y, x, z, indexing="ij")
                Y, X, Z = Y.ravel(), X.ravel(), Z.ravel()
            dist_srcs2 = np.zeros((ny * nx * nz, ns))
            dist_recs2 = np.zeros((ny * nx * nz, nr))
            for isrc, src in enumerate(srcs.T):
                dist_srcs2[:, isrc] = (X - src[0 + shiftdim]) ** 2 + (Z - src[1 + shiftdim]) ** 2
                if ndims == 3:
                    dist_srcs2[:, isrc] += (Y - src[0]) ** 2
            for irec, rec in enumerate(recs.T):
                dist_recs2[:, irec] = (X - rec[0 + shiftdim]) ** 2 + (Z - rec[1 + shiftdim]) ** 2
                if ndims == 3:
                    dist_recs2[:, irec] += (Y - rec[0]) ** 2
            trav_srcs = np.sqrt(dist_srcs2) / vel
            trav_recs = np.sqrt(dist_recs2) / vel
            dist_srcs = trav_srcs * vel
            dist_recs = trav_recs * vel
        elif mode == "eikonal":
            vel = np.asarray(vel, dtype=np.float64)
            if vel.shape != tuple(dims):
                raise ValueError(f"vel must have shape {tuple(dims)} for mode=eikonal")
            trav_srcs, dist_srcs = Kirchhoff._eikonal(srcs, vel, dims, dsamp, origin)
            trav_recs, dist_recs = Kirchhoff._eikonal(recs, vel, dims, dsamp, origin)
        else:
            raise NotImplementedError("method must be analytic or eikonal")
        trav_srcs_grad = np.gradient(trav_srcs.reshape(*dims, ns), *dsamp, axis=np.arange(ndims))
        trav_recs_grad = np.gradient(trav_recs.reshape(*dims, nr), *dsamp, axis=np.arange(ndims))
        return trav_srcs, trav_recs, dist_srcs, dist_recs, trav_srcs_grad, trav_recs_grad

    @staticmethod
    def _eikonal(pts, vel, dims, dsamp, origin, nthreads: int = 0):
        idx = np.round((pts.T - origin) / dsamp).astype(np.int32)  # kirchhoff.py:613
        idx = np.ascontiguousarray(idx)
        n = int(np.prod(dims))
        trav = np.empty((n, idx.shape[0]))
        dist = np.empty((n, idx.shape[0]))
        d = np.ascontiguousarray(np.asarray(dims, dtype=np.int32))
        h = np.ascontiguousarray(np.asarray(dsamp, dtype=np.float64))
        v = np.ascontiguousarray(vel, dtype=np.float64)
        _native.check(_native.lib().kgb_eikonal_tables(len(dims), _native.iptr(d), _native.dptr(h),
                                                       _native.dptr(v), idx.shape[0], _native.iptr(idx),
                                                       _native.dptr(trav), _native.dptr(dist), 2, nthreads))
        return trav, dist

    def _wavelet_reshaping(self, wav, dt, dimsrc, dimrec, dimv):
        """``wavfilter=True`` (``kirchhoff.py:659-681``): the omega factor of
        the wave equation applied to the wavelet's spectrum -- sqrt(j omega)
        for a 2-D model, -j omega for a 3-D model with 3-D sources and
        receivers; 2.5-D (2-D points in a 3-D model) is not available."""
        n = len(wav)
        jw = 2j * np.pi * np.fft.rfftfreq(n, dt)
        if dimv == 3 and 2 in (dimsrc, dimrec):
            raise NotImplementedError("2.D wavelet currently not available")
        factor = np.sqrt(jw) if (dimv == 2 and dimsrc == 2) else -jw
        return np.fft.irfft(factor * np.fft.rfft(wav, n=n), n=n)
