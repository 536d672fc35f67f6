"""Device-resident CGLS/LSQR against the reference solvers' iterates (golden
vectors from pylops.optimization.basic.cgls/lsqr) and the LSM workflow of the
reference's test_lsm.py.

Tolerances: the solvers keep float32 vectors and float64 scalars, the
reference keeps float64 vectors, so iterates and residual histories are held
to 1e-4 relative (12 iterations on a well-conditioned 240-unknown problem).
"""

import numpy as np
import pytest

from tests.helpers import kwargs_from_golden, load, rel

pytestmark = pytest.mark.gpu


def _op():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = kwargs_from_golden(load("k2d_dyn_noap"))
    return Kirchhoff(*args, engine="cuda", dtype="float32", **kw)


def test_lsqr_tracks_reference_iterates():
    from pylops_gb300.optimization import lsqr

    g = load("solvers")
    K = _op()
    its = []
    out = lsqr(K, g["d"].astype(np.float32), niter=12, callback=lambda x: its.append(np.array(x).copy()))
    x, istop, iiter, r1, r2, anorm, acond, arnorm, xnorm, var, cost = out
    assert iiter == int(g["lsqr_iiter"]) and istop == int(g["lsqr_istop"])
    ref_its = g["lsqr_iterates"].reshape(len(its), -1)
    for k in range(len(its)):
        assert rel(its[k], ref_its[k]) < 1e-4, (k, rel(its[k], ref_its[k]))
    assert rel(x, g["lsqr_x"]) < 1e-4
    np.testing.assert_allclose(cost, g["lsqr_cost"], rtol=1e-4)
    for val, key in ((r1, "lsqr_r1"), (r2, "lsqr_r2"), (anorm, "lsqr_anorm"), (acond, "lsqr_acond"),
                     (arnorm, "lsqr_arnorm"), (xnorm, "lsqr_xnorm")):
        np.testing.assert_allclose(val, float(g[key]), rtol=2e-3, err_msg=key)


def test_lsqr_graph_and_stepwise_paths_agree_bitwise():
    """run() replays the captured iteration inside one CUDA-graph WHILE node;
    with a callback it steps from the host.  Same kernels, same order."""
    from pylops_gb300.optimization import lsqr

    g = load("solvers")
    K = _op()
    d = g["d"].astype(np.float32)
    a = lsqr(K, d, niter=12)
    b = lsqr(K, d, niter=12, callback=lambda x: None)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(a[10], b[10])


def test_cgls_tracks_reference_iterates():
    from pylops_gb300.optimization import cgls

    g = load("solvers")
    K = _op()
    its = []
    x, istop, iiter, r1, r2, cost = cgls(K, g["d"].astype(np.float32), niter=12, tol=1e-10,
                                         callback=lambda x: its.append(np.array(x).copy()))
    assert iiter == int(g["cgls_iiter"])
    ref_its = g["cgls_iterates"].reshape(len(its), -1)
    for k in range(len(its)):
        assert rel(its[k], ref_its[k]) < 1e-4, (k, rel(its[k], ref_its[k]))
    np.testing.assert_allclose(cost, g["cgls_cost"], rtol=1e-4)
    xg, *_ = cgls(K, g["d"].astype(np.float32), niter=12, tol=1e-10)
    assert np.array_equal(xg, x)


def test_damped_solvers_match_reference():
    from pylops_gb300.optimization import cgls, lsqr

    g = load("solvers")
    K = _op()
    d = g["d"].astype(np.float32)
    out = lsqr(K, d, niter=6, damp=0.1)
    assert rel(out[0], g["lsqrd_x"]) < 1e-4
    np.testing.assert_allclose(out[10], g["lsqrd_cost"], rtol=1e-4)
    out = cgls(K, d, x0=0.1 * np.ones(K.ni, np.float32), niter=6, damp=0.1, tol=1e-10)
    assert rel(out[0], g["cglsd_x"]) < 1e-4
    np.testing.assert_allclose(out[5], g["cglsd_cost"], rtol=1e-4)


def test_generic_solver_path_matches_device_path():
    """A scaled operator goes through the generic (host-loop) path."""
    import torch

    from pylops_gb300.optimization import lsqr

    g = load("solvers")
    K = _op()
    d = torch.as_tensor(g["d"].astype(np.float32), device="cuda")
    a = lsqr(K, d, niter=8)[0]
    b = lsqr(1.0 * K, d, niter=8)[0]
    assert a.is_cuda and b.is_cuda
    assert rel(b.cpu().numpy(), a.cpu().numpy()) < 1e-5


def test_lsm_two_reflectors_like_reference_test():
    """pytests/test_lsm.py:79-106 with the device LSQR and scipy's lsqr."""
    from scipy.sparse.linalg import lsqr as sp_lsqr

    from pylops_gb300.optimization import lsqr
    from pylops_gb300.utils.wavelets import ricker
    from pylops_gb300.waveeqprocessing import LSM

    nx, nz, nt = 12, 20, 50
    x = np.arange(nx) * 1.0
    z = np.arange(nz) * 2.0
    t = np.arange(nt) * 0.004
    s2d = np.vstack((np.linspace(x.min(), x.max(), 6), 2 * np.ones(6)))
    r2d = np.vstack((np.linspace(x.min(), x.max(), 4), 2 * np.ones(4)))
    wav, _, wavc = ricker(t[:21], f0=40)
    refl = np.zeros((nx, nz))
    refl[:, nz // 2] = 1
    refl[:, 3 * nz // 4] = 1
    for dynamic in (False, True):
        lsm = LSM(z, x, t, s2d, r2d, 500.0, wav, wavc, mode="analytic", dynamic=dynamic, dottest=True,
                  dtype="float32")
        d = (lsm.Demop * refl.ravel().astype(np.float32)).reshape(6, 4, nt)
        for solver, kw in ((sp_lsqr, dict(iter_lim=100)), (lsqr, dict(niter=100))):
            minv = lsm.solve(d.ravel(), solver=solver, **kw)
            dinv = (lsm.Demop * minv.ravel().astype(np.float32)).reshape(6, 4, nt)
            np.testing.assert_array_almost_equal(d / d.max(), dinv / d.max(), decimal=2)
            np.testing.assert_array_almost_equal(refl / refl.max(), minv / refl.max(), decimal=1)


def test_right_preconditioned_lsqr_with_warm_start_tracks_reference():
    """lsqr(Kop * Diagonal(p), d, x0=z0) runs on the device path (the diagonal
    is folded into the captured iteration) and follows the reference's
    iterates; the generic host-loop path on a scaled copy agrees."""
    import torch

    from pylops_gb300.basicoperators import Diagonal
    from pylops_gb300.optimization import lsqr
    from pylops_gb300.optimization.cls_basic import _is_device_kirchhoff

    g = load("solvers_precond")
    K = _op()
    Op = K * Diagonal(g["p"].astype(np.float32), dtype="float32")
    assert _is_device_kirchhoff(Op)
    its = []
    d = g["d"].astype(np.float32)
    z0 = g["z0"].astype(np.float32)
    out = lsqr(Op, d, x0=z0, niter=10, atol=0.0, btol=1e-3, callback=lambda x: its.append(np.array(x).copy()))
    assert out[2] == int(g["iiter"]) and out[1] == int(g["istop"])
    for k in range(len(its)):
        assert rel(its[k], g["iterates"][k]) < 1e-4, (k, rel(its[k], g["iterates"][k]))
    np.testing.assert_allclose(out[10], g["cost"], rtol=1e-4)
    graph = lsqr(Op, d, x0=z0, niter=10, atol=0.0, btol=1e-3)
    assert np.array_equal(graph[0], out[0])
    generic = lsqr(1.0 * Op, torch.as_tensor(d, device="cuda"), x0=torch.as_tensor(z0, device="cuda"), niter=10,
                   atol=0.0, btol=1e-3)[0]
    assert rel(generic.cpu().numpy(), out[0]) < 1e-4
