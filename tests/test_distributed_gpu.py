"""The source-sharded operator, CGLS and LSQR with the CUDA Kirchhoff as each
rank's local operator: two gloo ranks (host collectives; no kernel of one
rank waits on the other) share cuda:0, each holding the tables of its half
of the sources.  Sharded forward = the unsharded operator's rows, sharded
adjoint = the unsharded image, distributed CGLS/LSQR = the single-process
device solvers.

Tolerances: each rank's operator is float32 with its own fixed-point scale
(its own sources' largest weight) and its own gather order, so the sharded
applications agree with the unsharded ones to 1e-6 relative; the solvers
(float32 vectors, float64 scalars) to 1e-4 over 8 iterations.
"""

import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, errfile):
    import torch
    import torch.distributed as dist

    from oracle.kirchhoff_oracle import ricker
    from pylops_gb300.distributed import DistributedKirchhoff, cgls, lsqr, source_shard
    from pylops_gb300.optimization import cgls as dev_cgls, lsqr as dev_lsqr
    from pylops_gb300.waveeqprocessing import Kirchhoff

    torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        nz, nx, ns, nr, nt = 50, 80, 6, 20, 300
        z, x, t = np.arange(nz) * 4.0, np.arange(nx) * 4.0, np.arange(nt) * 0.004
        srcs = np.vstack((np.linspace(x[0], x[-1], ns), np.zeros(ns)))
        recs = np.vstack((np.linspace(x[0], x[-1], nr), np.zeros(nr)))
        wav, _, wc = ricker(t[:41], f0=20)
        kw = dict(mode="analytic", dynamic=True, angleaperture=60.0, engine="cuda", dtype="float32")
        full = Kirchhoff(z, x, t, srcs, recs, 2000.0, wav, wc, **kw)
        s0, s1 = source_shard(ns, rank, world)
        local = Kirchhoff(z, x, t, srcs[:, s0:s1], recs, 2000.0, wav, wc, **kw)
        D = DistributedKirchhoff(local)
        rows = slice(s0 * nr * nt, s1 * nr * nt)
        rng = np.random.default_rng(0)
        m = rng.standard_normal(full.ni).astype(np.float32)
        d = rng.standard_normal(full.shape[0]).astype(np.float32)
        rel = lambda a, b: float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))  # noqa: E731
        assert rel(D.matvec(m), (full @ m)[rows]) < 1e-6
        assert rel(D.rmatvec(d[rows]), full.H @ d) < 1e-6
        refl = np.zeros((nx, nz), np.float32)
        refl[:, 20] = 1.0
        refl[:, 35] = -0.5
        y = full @ refl.ravel()
        xc = cgls(D, y[rows], niter=8, tol=0.0)
        xr = dev_cgls(full, y, niter=8, tol=0.0)
        assert rel(xc[0], xr[0]) < 1e-4
        np.testing.assert_allclose(xc[5], xr[5], rtol=1e-4)
        xl = lsqr(D, y[rows], niter=8)
        xlr = dev_lsqr(full, y, niter=8)
        assert xl[2] == xlr[2] and xl[1] == xlr[1]
        assert rel(xl[0], xlr[0]) < 1e-4
        np.testing.assert_allclose(xl[10], xlr[10], rtol=1e-4)
    except Exception as e:  # reported to the parent, which fails the test
        with open(f"{errfile}.{rank}", "w") as f:
            f.write(repr(e))
        raise
    finally:
        dist.destroy_process_group()


def test_two_ranks_share_the_gpu_with_sharded_cuda_operators(tmp_path):
    import torch.multiprocessing as mp

    errfile = str(tmp_path / "err")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env_path = os.environ.get("PYTHONPATH", "")
    os.environ["PYTHONPATH"] = root + (os.pathsep + env_path if env_path else "")
    mp.spawn(_rank_main, args=(2, _free_port(), errfile), nprocs=2, join=True)
    for r in range(2):
        assert not os.path.exists(f"{errfile}.{r}"), open(f"{errfile}.{r}").read()
