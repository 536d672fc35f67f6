"""Full-size workloads: the 2-D eikonal dynamic workload (300x800, 64x400
traces, nt=1501), the 3-D analytic dynamic workload (100x100x120, 16x400
traces, nt=1001) and the learned-LSM operator (256x512, 48x256, nt=1201).

At these sizes the float64 oracle cannot run whole in a test, so parity is
checked on sampled sources (forward traces of those sources; adjoint of data
that is zero outside them), and the rest through size-independent
properties: adjointness with float64 dot products, linearity and bitwise
determinism.  Tolerance: 1e-5 relative L2 against float64."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _workload2d():
    from bench import build_operator, make_workload

    w = make_workload()
    K, _ = build_operator(w)
    return K


def _workload3d():
    from pylops_gb300.utils.wavelets import ricker
    from pylops_gb300.waveeqprocessing import Kirchhoff

    ny = nx = 100
    nz = 120
    y, x, z = np.arange(ny) * 10.0, np.arange(nx) * 10.0, np.arange(nz) * 10.0
    t = np.arange(1001) * 0.004
    wav, _, wc = ricker(t[:41], f0=20)
    sy, sx = np.meshgrid(np.linspace(y[0], y[-1], 4), np.linspace(x[0], x[-1], 4), indexing="ij")
    ry, rx = np.meshgrid(np.linspace(y[0], y[-1], 20), np.linspace(x[0], x[-1], 20), indexing="ij")
    srcs = np.vstack((sy.ravel(), sx.ravel(), np.zeros(16)))
    recs = np.vstack((ry.ravel(), rx.ravel(), np.zeros(400)))
    return Kirchhoff(z, x, t, srcs, recs, 2500.0, wav, wc, y=y, mode="analytic", dynamic=True,
                     engine="cuda", dtype="float32")


def _workload_lsm():
    from pylops_gb300.learned.experiment import lsm_operator

    return lsm_operator()


def _dot(a, b):
    return float(torch.dot(a.double(), b.double()))


def _check(K, sources, seed=0):
    from bench import _cpu_step, _padded_wavelet
    from oracle.kirch_oracle_c import COracle, build

    build()
    g = torch.Generator(device="cuda").manual_seed(seed)
    m = torch.randn(K.ni, device="cuda", generator=g)
    d = torch.randn(K.shape[0], device="cuda", generator=g)
    y1 = torch.empty(K.shape[0], device="cuda")
    y2 = torch.empty_like(y1)
    x1 = torch.empty(K.ni, device="cuda")
    x2 = torch.empty_like(x1)
    for v in (0, 1):
        K.set_spread_variant(v)
        K.apply_into(m, y1)
        K.apply_into(m, y2)
        assert torch.equal(y1, y2), f"forward variant {v} not bitwise repeatable"
    K.apply_into(d, x1, adjoint=True)
    K.apply_into(d, x2, adjoint=True)
    assert torch.equal(x1, x2), "adjoint not bitwise repeatable"
    # adjointness and linearity
    lhs, rhs = _dot(y1, d), _dot(m, x1)
    assert abs(lhs - rhs) / max(abs(lhs), abs(rhs)) < 1e-4
    K.apply_into((2.5 * m).contiguous(), y2)
    assert float(torch.linalg.norm(y2 - 2.5 * y1) / torch.linalg.norm(2.5 * y1)) < 1e-5
    # parity against the float64 C oracle on sampled sources
    C = COracle(K, _padded_wavelet(K))
    mh = m.cpu().numpy().astype(np.float64)
    dh = d.cpu().numpy().astype(np.float64).reshape(K.nsnr, K.nt)
    for s in sources:
        rows = slice(s * K.nr, (s + 1) * K.nr)
        yc, xc = _cpu_step(C, mh, dh, s, s + 1)
        yg = y1.view(K.nsnr, K.nt)[rows].cpu().numpy()
        ef = np.linalg.norm(yg - yc[rows]) / np.linalg.norm(yc[rows])
        assert ef < 1e-5, f"source {s}: forward error {ef:.2e}"
        dz = torch.zeros(K.nsnr, K.nt, device="cuda")
        dz[rows] = d.view(K.nsnr, K.nt)[rows]
        K.apply_into(dz.view(-1), x2, adjoint=True)
        xg = x2.cpu().numpy()
        ea = np.linalg.norm(xg - xc) / np.linalg.norm(xc)
        assert ea < 1e-5, f"source {s}: adjoint error {ea:.2e}"


def test_2d_eikonal_dynamic_workload_full_size():
    K = _workload2d()
    _check(K, sources=(0, 37))


def test_3d_analytic_dynamic_workload_full_size():
    K = _workload3d()
    assert K.ni == 100 * 100 * 120 and K.nsnr == 16 * 400
    _check(K, sources=(5,))


def test_learned_lsm_operator_full_size():
    K = _workload_lsm()
    _check(K, sources=(0, 30))
