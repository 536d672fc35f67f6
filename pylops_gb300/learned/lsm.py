"""Learned-preconditioned least-squares migration.

A :class:`~pylops_gb300.learned.unet.UNet` maps the migrated image
``K^H d`` to an estimate of the reflectivity; it is trained on pairs that
the Kirchhoff operator itself generates from random reflectivity models
(:func:`random_reflectivity`, :func:`make_pairs`, :func:`train`).  Because
LSQR needs a linear operator, the network is used as a **warm start**:
``x0 = alpha UNet(K^H d)`` with ``alpha`` the least-squares fit of
``K x0`` to the data, together with an optional fixed linear **right
preconditioner** ``P = diag(p)`` (:func:`illumination_diagonal`, the
inverse square root of the diagonal of ``K^H K``), and LSQR
(``pylops/optimization/cls_basic.py:711-1351``) runs on ``K P`` from
``z0 = x0 / p`` until the data residual reaches ``tol ||d||``.  Plain LSQR
from zero is both the fallback (used when the warm start does not lower the
residual) and the measure of the result (data residual and model error).

PyLops has no counterpart of the network; the surrounding solve is the
reference's ``lsqr(Kop * Diagonal(p), d, x0=z0)``.
"""

from __future__ import annotations

import math
import sys
import time
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .. import _native
from .unet import UNet

__all__ = ["random_reflectivity", "make_pairs", "make_residual_pairs", "train", "illumination_diagonal",
           "point_spread_functions", "LearnedLSM", "SolveInfo"]


def random_reflectivity(nx: int, nz: int, rng: np.random.Generator, dx: float = 5.0, dz: float = 5.0,
                        nlayers=(3, 15), nfaults=(0, 3), spike_density=(1e-4, 1e-3), max_dip: float = 20.0,
                        max_throw: float = 40.0, spike_std: float = 0.1) -> np.ndarray:
    """Seeded layered reflectivity (nx, nz): ``nlayers`` interfaces (inclusive
    range) with dips U[-max_dip, max_dip] degrees between layers of impedance
    U[1.5, 4.5], cut by ``nfaults`` planar faults (dip U[60, 90] degrees,
    throw U[-max_throw, max_throw] m), reflectivity (I[z+1]-I[z])/(I[z+1]+I[z]),
    plus N(0, spike_std^2) spikes at a density U[spike_density] of the
    pixels."""
    xs = np.arange(nx, dtype=np.float64)[:, None] * dx
    zs = np.arange(nz, dtype=np.float64)[None, :] * dz
    Z = nz * dz
    xc = 0.5 * nx * dx
    nl = int(rng.integers(nlayers[0], nlayers[1] + 1))
    z0 = np.sort(rng.uniform(0.04 * Z, 0.96 * Z, nl))
    slope = np.tan(np.deg2rad(rng.uniform(-max_dip, max_dip, nl)))
    imp = rng.uniform(1.5, 4.5, nl + 1)
    # depth at which each pixel reads the layered model (shifted across faults)
    zz = np.broadcast_to(zs, (nx, nz)).copy()
    for _ in range(int(rng.integers(nfaults[0], nfaults[1] + 1))):
        xf = rng.uniform(0.15, 0.85) * nx * dx
        phi = np.deg2rad(rng.uniform(60.0, 90.0)) * (1 if rng.random() < 0.5 else -1)
        throw = rng.uniform(-max_throw, max_throw)
        side = (xs - xf - (zs - 0.5 * Z) / np.tan(phi)) > 0
        zz -= throw * side
    layer = np.zeros((nx, nz), dtype=np.int64)
    for k in range(nl):
        layer += (z0[k] + slope[k] * (xs - xc)) < zz
    I = imp[layer]
    r = np.zeros((nx, nz))
    r[:, :-1] = (I[:, 1:] - I[:, :-1]) / (I[:, 1:] + I[:, :-1])
    ns = int(round(rng.uniform(*spike_density) * nx * nz))
    if ns:
        idx = rng.choice(nx * nz, size=ns, replace=False)
        r.reshape(-1)[idx] += spike_std * rng.standard_normal(ns)
    return r.astype(np.float32)


def _normalised(m: np.ndarray) -> np.ndarray:
    s = float(np.sqrt(np.mean(np.asarray(m, np.float64) ** 2)))
    return (m / s).astype(np.float32) if s > 0 else m.astype(np.float32)


def make_pairs(op, n: int, seed: int = 0, generator=random_reflectivity, **kw):
    """``n`` training pairs ``(K^H K m, m / rms(m))`` as float32 CUDA tensors
    of shape (n, nx, nz), the models drawn by ``generator`` with a
    ``default_rng(seed)``; forward and adjoint run on the current stream."""
    import torch

    nx, nz = op.dims
    rng = np.random.default_rng(seed)
    X = torch.empty((n, nx, nz), dtype=torch.float32, device="cuda")
    M = torch.empty((n, nx, nz), dtype=torch.float32, device="cuda")
    d = torch.empty(op.shape[0], dtype=torch.float32, device="cuda")
    for i in range(n):
        m = _normalised(generator(nx, nz, rng, **kw))
        M[i].copy_(torch.from_numpy(m), non_blocking=False)
        op.apply_into(M[i].reshape(-1), d)
        op.apply_into(d, X[i].reshape(-1), adjoint=True)
    return X, M


def make_residual_pairs(op, net: UNet, n: int, seed: int = 1, generator=random_reflectivity, **kw):
    """Second-stage pairs for the network steps of the solve: for a fresh
    model m with data d = K m, the network's warm start x1 = alpha UNet(K^H d)
    (alpha the least-squares fit of K x1 to d) leaves the error e = m - x1;
    the pair is (K^H K e, e / rms(e)) -- the gradient the solve feeds the
    network after its warm start, and what the network should return.
    Float32 CUDA tensors (n, nx, nz)."""
    import torch

    nx, nz = op.dims
    rng = np.random.default_rng(seed)
    X = torch.empty((n, nx, nz), dtype=torch.float32, device="cuda")
    E = torch.empty((n, nx, nz), dtype=torch.float32, device="cuda")
    d = torch.empty(op.shape[0], dtype=torch.float32, device="cuda")
    ku = torch.empty_like(d)
    img = torch.empty(op.ni, dtype=torch.float32, device="cuda")
    for i in range(n):
        m = torch.from_numpy(_normalised(generator(nx, nz, rng, **kw))).to("cuda").reshape(-1)
        op.apply_into(m, d)
        op.apply_into(d, img, adjoint=True)
        u = net.forward(img.view(nx, nz)).reshape(-1).contiguous()
        op.apply_into(u, ku)
        kk = float(torch.dot(ku.double(), ku.double()))
        alpha = float(torch.dot(ku.double(), d.double())) / kk if kk > 0 else 0.0
        e = m - alpha * u
        rms = float(torch.sqrt(torch.mean(e.double() ** 2)))
        E[i] = (e / rms if rms > 0 else e).view(nx, nz)
        op.apply_into(e.contiguous(), d)
        op.apply_into(d, X[i].reshape(-1), adjoint=True)
    return X, E


def train(net: UNet, X, M, steps: int, batch: int = 8, lr: float = 1e-3, lr_final: float = 1e-4, seed: int = 0,
          log_every: int = 0) -> List[float]:
    """Adam on random mini-batches of (X, M) with a cosine learning-rate
    decay from ``lr`` to ``lr_final``; returns the loss of every step (read
    back once at the end, so the steps run without host synchronisation)."""
    import torch

    n = X.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = torch.empty(steps, dtype=torch.float64, device="cuda")
    for k in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g).to("cuda")
        xb, mb = X.index_select(0, idx), M.index_select(0, idx)
        cur = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * k / max(steps - 1, 1)))
        losses[k] = net.train_step(xb, mb, lr=cur)
        if log_every and (k % log_every == 0 or k == steps - 1):
            print(f"step {k:5d} lr {cur:.2e} loss {float(losses[k]):.4f}", file=sys.stderr, flush=True)
    net.check_errors()
    return losses.cpu().tolist()


def illumination_diagonal(op, eps: float = 1e-3) -> np.ndarray:
    """Right preconditioner ``p = 1/sqrt(diag(K^H K) + eps max diag)`` of a
    dynamic 2-D Kirchhoff operator.  Every trace holds one wavelet per image
    point, so ``||K e_i||^2 = sum_{s,r} w_{s,r,i}^2 E`` (E the wavelet energy
    after linear interpolation, averaged over the fraction) with
    ``w = 2 cos((a_s - a_r)/2) A_s A_r / v`` (``kirchhoff.py:820-889``);
    ``4 cos^2((a-b)/2) = 2 (1 + cos a cos b + sin a sin b)`` splits the double
    sum into per-source and per-receiver sums, O(ni (ns + nr)).  The angle
    taper is included, the offset aperture gate and the time-window cut are
    not.  Returns float32 (ni,)."""
    if not op.dynamic:
        return np.ones(op.ni, dtype=np.float32)

    def sums(amp, ang):
        amp = np.asarray(amp, np.float64)
        ang = np.asarray(ang, np.float64)
        amin, amax = op.angleaperture
        a = np.abs(ang)
        tap = np.where(a < amax, 1.0, 0.0)
        mid = (a >= amin) & (a < amax)
        if np.any(mid):
            itap = np.floor(20 * (a[mid] - amin) / (amax - amin)).astype(int).clip(0, 20)
            tap[mid] = np.asarray(op.aperturetap)[itap]
        w = (amp * tap) ** 2
        return w.sum(1), (w * np.cos(ang)).sum(1), (w * np.sin(ang)).sum(1)

    S0, Sc, Ss = sums(op.amp_srcs, op.angle_srcs)
    R0, Rc, Rs = sums(op.amp_recs, op.angle_recs)
    vel = np.asarray(op.vel, np.float64).reshape(-1) * np.ones(op.ni)
    # energy of (1-f) wav(t) + f wav(t-1) averaged over the interpolation
    # fraction f in [0, 1): (2 sum wav^2 + sum wav(t) wav(t+1)) / 3
    w = np.asarray(op.wav, np.float64).ravel()
    ew = float(2.0 * np.dot(w, w) + np.dot(w[1:], w[:-1])) / 3.0
    diag = 2.0 / vel ** 2 * (S0 * R0 + Sc * Rc + Ss * Rs) * ew
    diag = np.maximum(diag, 0.0)
    return (1.0 / np.sqrt(diag + eps * diag.max())).astype(np.float32)


def point_spread_functions(op, psfx, psfz, psfsize=(31, 31)):
    """Point-spread functions of the Hessian ``K^H K`` of a 2-D Kirchhoff
    operator, the filters of an image-domain Hessian
    (``NonStationaryConvolve2D``): unit scatterers at the grid ``psfx`` x
    ``psfz`` (indices), one forward and one adjoint, and a ``psfsize``
    window around each scatterer (the workflow of ``tutorials/ilsm.py``).
    The grid spacing must exceed the window so windows do not overlap.
    Returns a float32 CUDA tensor (len(psfx), len(psfz), *psfsize)."""
    import torch

    nx, nz = op.dims
    hx, hz = psfsize
    psfx, psfz = np.asarray(psfx), np.asarray(psfz)
    if np.any(np.diff(psfx) < hx) or np.any(np.diff(psfz) < hz):
        raise ValueError("point scatterers closer than the PSF window")
    if psfx.min() < hx // 2 or psfz.min() < hz // 2 or psfx.max() + hx // 2 >= nx or psfz.max() + hz // 2 >= nz:
        raise ValueError("PSF windows must lie inside the image")
    m = torch.zeros((nx, nz), dtype=torch.float32, device="cuda")
    m[torch.as_tensor(psfx, device="cuda")[:, None], torch.as_tensor(psfz, device="cuda")[None, :]] = 1.0
    d = torch.empty(op.shape[0], dtype=torch.float32, device="cuda")
    img = torch.empty(op.ni, dtype=torch.float32, device="cuda")
    op.apply_into(m.reshape(-1), d)
    op.apply_into(d, img, adjoint=True)
    img = img.view(nx, nz)
    hs = torch.empty((len(psfx), len(psfz), hx, hz), dtype=torch.float32, device="cuda")
    for i, px in enumerate(psfx):
        for j, pz in enumerate(psfz):
            hs[i, j] = img[px - hx // 2:px + hx // 2 + 1, pz - hz // 2:pz + hz // 2 + 1]
    return hs


@dataclass
class SolveInfo:
    """Outcome of one solve: LSQR iterations, wall time (s, device-
    synchronised), final relative data residual ||d - K x|| / ||d||
    (recomputed), the LSQR stopping code, the number of network directions
    used (warm start included), the relative residual after them, operator
    pairs (one forward + one adjoint) spent in total, and the LSQR residual
    history."""
    iterations: int
    seconds: float
    residual: float
    istop: int
    network_steps: int = 0
    network_residual: float = 1.0
    operator_pairs: int = 0
    gpu_launches: int = 0
    cost: List[float] = field(default_factory=list)


class LearnedLSM:
    """Network-accelerated LSQR on a Kirchhoff operator.

    ``solve(d, tol)`` reaches a data residual below ``tol ||d||`` in up to
    three phases:

    1. **warm start** -- ``p_0 = UNet(K^H d)``;
    2. **network steps** -- ``p_j = UNet(K^H r_{j-1})``: the gradient
       ``K^H r = K^H K e`` has the form of the training inputs, so the
       network maps it to an estimate of the error ``e``.  After each
       direction the model is the minimum-residual combination
       ``x = sum_j c_j p_j`` (``c`` from the Gram system of the ``K p_j``, a
       flexible Krylov step).  The phase ends when a direction lowers the
       residual by less than the factor ``step_ratio`` (that direction is
       dropped), after ``steps`` directions, or at ``tol``;
    3. **LSQR** (``cls_basic.py:711-1351``) on ``K`` (or ``K diag(p)`` with a
       right preconditioner) from the network model, with ``btol`` rescaled
       so that it stops at ``tol ||d||`` (``atol = 0``).

    ``net=None`` gives plain LSQR from zero, which is also the fallback when
    the warm start does not lower the residual."""

    def __init__(self, op, net: Optional[UNet] = None, diag: Optional[np.ndarray] = None, steps: int = 4,
                 step_ratio: float = 0.7, psf=None, psf_iters: int = 10):
        import torch

        self.op = op
        self.net = net
        self.psf = psf  # image-domain Hessian (NonStationaryConvolve2D): classical warm start
        self.psf_iters = int(psf_iters)
        self.steps = int(steps)
        self.step_ratio = float(step_ratio)
        self.diag = None if diag is None else np.ascontiguousarray(diag, dtype=np.float32)
        self._diag_dev = None if diag is None else torch.as_tensor(self.diag, device="cuda")
        self._dots_dev = torch.empty(32, dtype=torch.float64, device="cuda")

    # ------------------------------------------------------------ helpers
    def _dots(self, pairs) -> List[float]:
        """float64 inner products of float32 device vectors, one readback."""
        import torch

        s = torch.cuda.current_stream().cuda_stream
        L = _native.lib()
        for k, (a, b) in enumerate(pairs):
            _native.check(L.kgb_dot_f64(a.data_ptr(), b.data_ptr(), a.numel(), self._dots_dev[k:].data_ptr(), s))
        return self._dots_dev[:len(pairs)].cpu().tolist()

    @staticmethod
    def _lincomb(out, base, c0: float, vecs, coefs) -> None:
        import ctypes

        import torch

        k = len(vecs)
        ptrs = (ctypes.c_void_p * max(k, 1))(*[v.data_ptr() for v in vecs])
        cs = (ctypes.c_double * max(k, 1))(*[float(c) for c in coefs])
        _native.check(_native.lib().kgb_lincomb_f32(out.data_ptr(), None if base is None else base.data_ptr(),
                                                    float(c0), ptrs, cs, k, out.numel(),
                                                    torch.cuda.current_stream().cuda_stream))

    def network_phase(self, d, tol: float):
        """Phases 1-2.  Returns ``(x, rel, ndirections, operator_pairs)``;
        x is None (and rel 1) when the warm start does not lower the
        residual."""
        import torch

        op = self.op
        nx, nz = op.dims
        dd = self._dots([(d, d)])[0]
        if dd <= 0:
            return None, 1.0, 0, 0
        g = torch.empty(op.ni, dtype=torch.float32, device="cuda")
        r = torch.empty_like(d)
        P, Q = [], []
        nmax = 1 + max(self.steps, 0)
        G = np.zeros((nmax, nmax))
        b = np.zeros(nmax)
        c = np.zeros(0)
        rel = 1.0
        pairs = 0
        info = op.info()
        fa = info["kernels_forward"] + info["kernels_adjoint"]
        self._launches = 1  # the |d|^2 dot
        src = d
        for j in range(nmax):
            op.apply_into(src, g, adjoint=True)
            l0 = self.net.launches
            p = self.net.forward(g.view(nx, nz)).reshape(-1).contiguous()
            self._launches += self.net.launches - l0
            q = torch.empty_like(d)
            op.apply_into(p, q)
            pairs += 1
            self._launches += fa + len(Q) + 2
            vals = self._dots([(q, v) for v in Q] + [(q, q), (q, d)])
            G[j, :j] = G[:j, j] = vals[:j]
            G[j, j] = vals[j]
            b[j] = vals[j + 1]
            if G[j, j] <= 0:
                break
            cj = np.linalg.lstsq(G[:j + 1, :j + 1], b[:j + 1], rcond=1e-10)[0]
            relj = math.sqrt(max(dd - float(b[:j + 1] @ cj), 0.0) / dd)
            if relj > rel * (1.0 if j == 0 else self.step_ratio):
                break  # this direction does not pay: keep the previous combination
            P.append(p)
            Q.append(q)
            c, rel = cj, relj
            if rel <= tol or j == nmax - 1:
                break
            self._lincomb(r, d, 1.0, Q, -c)  # r = d - sum c_j K p_j
            self._launches += 1
            src = r
        if not P:
            return None, 1.0, 0, pairs
        x = torch.empty(op.ni, dtype=torch.float32, device="cuda")
        self._lincomb(x, None, 0.0, P, c)
        self._launches += 1
        return x, rel, len(P), pairs

    def psf_phase(self, d):
        """Classical warm start: CGLS on the image-domain Hessian
        (``psf``, ``psf_iters`` iterations) from the migrated image, scaled by
        the least-squares fit of its data to d.  Returns (x0 or None, rel,
        operator pairs)."""
        import torch

        from ..optimization.basic import cgls

        op = self.op
        img = torch.empty(op.ni, dtype=torch.float32, device="cuda")
        op.apply_into(d, img, adjoint=True)
        u = cgls(self.psf, img, niter=self.psf_iters, tol=0.0)[0].contiguous()
        info = op.info()
        self._launches += info["kernels_adjoint"] + 2 * self.psf_iters + info["kernels_forward"]
        Ku = torch.empty_like(d)
        op.apply_into(u, Ku)
        kd, kk, dd = self._dots([(Ku, d), (Ku, Ku), (d, d)])
        self._launches += 3
        if kk <= 0 or dd <= 0:
            return None, 1.0, 1
        alpha = kd / kk
        rel = math.sqrt(max(dd - alpha * kd, 0.0) / dd)
        if rel >= 1.0:
            return None, 1.0, 1
        return u.mul_(alpha), rel, 1

    def solve(self, d, tol: float = 1e-2, niter: int = 500, use_net: bool = True) -> tuple:
        """Returns ``(x, SolveInfo)``.  ``d`` is a CUDA tensor (x is then a
        float32 CUDA tensor) or a host array (staged through pinned memory
        inside the timed region; x is then a numpy array)."""
        import torch

        from ..basicoperators import Diagonal
        from ..optimization.cls_basic import LSQR

        op = self.op
        host = not torch.is_tensor(d)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if host:  # host data: pinned staging copy inside the timed region
            dd = torch.from_numpy(np.ascontiguousarray(d, dtype=np.float32).reshape(-1)).pin_memory().to(
                "cuda", non_blocking=True)
        else:
            dd = d.to(device="cuda", dtype=torch.float32).reshape(-1).contiguous()
        x0, rel0, nsteps, pairs = None, 1.0, 0, 0
        self._launches = 0
        if use_net and self.net is not None:
            x0, rel0, nsteps, pairs = self.network_phase(dd, tol)
        elif use_net and self.psf is not None:
            x0, rel0, pairs = self.psf_phase(dd)
        launches = self._launches
        iiter, istop, cost = 0, 1, [rel0]
        x = x0
        if rel0 > tol:
            Op = op if self._diag_dev is None else op * Diagonal(self.diag, dtype="float32")
            z0 = x0
            if x0 is not None and self._diag_dev is not None:
                z0 = x0 / self._diag_dev
            z, istop, iiter, _r1, *_rest, cost = LSQR(Op).solve(dd, x0=z0, atol=0.0, btol=tol / rel0, conlim=1e8,
                                                                niter=niter, calc_var=False)
            x = z if self._diag_dev is None else z * self._diag_dev
            pairs += int(iiter) + 1
            info = op.info()
            F = info["kernels_forward"] + (0 if self._diag_dev is None else 1)
            A = info["kernels_adjoint"] + (0 if self._diag_dev is None else 1)
            # setup: state, |u|, beta, scale, [K x0, subtract], K^H u, |v|, alfa, scale, copy, target;
            # one iteration: K v, u update, beta, scale, K^H u, v update, rotation, x/w update, tail
            launches += 10 + A + (F + 1 if x0 is not None else 0) + int(iiter) * (7 + F + A)
        if host:
            x = x.cpu().numpy()
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        if host:
            x = torch.as_tensor(x, device="cuda")
        kx = torch.empty_like(dd)
        op.apply_into(x.contiguous(), kx)
        r = torch.empty_like(dd)
        self._lincomb(r, kx, 1.0, [dd], [-1.0])
        rr, d2 = self._dots([(r, r), (dd, dd)])
        res = math.sqrt(rr / d2) if d2 > 0 else 0.0
        if host:
            x = x.cpu().numpy()
        return x, SolveInfo(int(iiter), secs, res, int(istop), nsteps, rel0, pairs, launches,
                            [float(v) for v in np.asarray(cost)])
