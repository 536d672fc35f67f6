"""Source-sharded operator, CGLS and LSQR with two gloo ranks on the CPU; each
rank's local operator is the float64 oracle of its sources (the GPU operator
takes its place on a GPU).  The sharded forward must reproduce the
unsharded rows, the adjoint the unsharded image, and CGLS and LSQR the
unsharded iterates, stopping reasons and norms, to float64 rounding."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, errfile):
    import torch.distributed as dist

    from oracle.kirchhoff_oracle import KirchhoffOracle, cgls as oracle_cgls, lsqr as oracle_lsqr
    from pylops_gb300.distributed import DistributedKirchhoff, cgls, lsqr, source_shard
    from pylops_gb300.linearoperator import LinearOperator
    from tests.helpers import kwargs_from_golden, load

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        g = load("k2d_dyn_noap")
        args, kw = kwargs_from_golden(g)
        full = KirchhoffOracle(*args, **kw)
        s0, s1 = source_shard(full.ns, rank, world)
        srcs = args[3][:, s0:s1]
        local = KirchhoffOracle(*args[:3], srcs, *args[4:], **kw)

        class _Op(LinearOperator):
            def __init__(self, o):
                super().__init__(dtype=np.float64, shape=o.shape)
                self.o = o

            def _matvec(self, x):
                return self.o.matvec(x)

            def _rmatvec(self, y):
                return self.o.rmatvec(y)

        D = DistributedKirchhoff(_Op(local))
        rows = slice(s0 * full.nr * full.nt, s1 * full.nr * full.nt)
        m = np.asarray(g["m_in"], np.float64)
        d = np.asarray(g["d_in"], np.float64)
        assert np.allclose(D.matvec(m), full.matvec(m)[rows], rtol=0, atol=1e-12)
        img = D.rmatvec(d[rows])
        ref = full.rmatvec(d)
        assert np.linalg.norm(img - ref) / np.linalg.norm(ref) < 1e-12
        y = full.matvec(m)
        x, istop, it, r1, r2, cost = cgls(D, y[rows], niter=6, tol=1e-12)
        xr, istop_r, it_r, r1_r, r2_r, cost_r, _ = oracle_cgls(full.matvec, full.rmatvec, y, full.ni, niter=6,
                                                                tol=1e-12)
        assert it == it_r and istop == istop_r
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-10
        assert np.allclose(cost, cost_r, rtol=1e-10)
        assert abs(r1 - r1_r) <= 1e-10 * abs(r1_r)
        # LSQR: the data-space norm is the one all-reduce per iteration
        out = lsqr(D, y[rows], niter=6)
        ref_l = oracle_lsqr(full.matvec, full.rmatvec, y, full.ni, niter=6)
        assert out[2] == ref_l[2] and out[1] == ref_l[1]
        assert np.linalg.norm(out[0] - ref_l[0]) / np.linalg.norm(ref_l[0]) < 1e-10
        assert np.allclose(out[10], ref_l[9], rtol=1e-10)
        for k in range(3, 9):  # r1norm, r2norm, anorm, acond, arnorm, xnorm
            assert abs(out[k] - ref_l[k]) <= 1e-9 * abs(ref_l[k]), (k, out[k], ref_l[k])
        # with damping and an early stop on atol/btol
        out = lsqr(D, y[rows], niter=50, damp=0.3, atol=1e-3, btol=1e-3)
        ref_l = oracle_lsqr(full.matvec, full.rmatvec, y, full.ni, niter=50, damp=0.3, atol=1e-3, btol=1e-3)
        assert out[2] == ref_l[2] and out[1] == ref_l[1] and out[1] != 0
        assert np.linalg.norm(out[0] - ref_l[0]) / np.linalg.norm(ref_l[0]) < 1e-9
    except Exception as e:  # report to the parent, which fails the test
        with open(f"{errfile}.{rank}", "w") as f:
            f.write(repr(e))
        raise
    finally:
        dist.destroy_process_group()


def test_source_shard_covers_every_source_once():
    from pylops_gb300.distributed import source_shard

    for ns in (1, 5, 6, 64, 65):
        for world in (1, 2, 3, 8):
            if world > ns:
                continue
            blocks = [source_shard(ns, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == ns
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
            assert max(b - a for a, b in blocks) - min(b - a for a, b in blocks) <= 1


def test_two_rank_sharded_operator_cgls_and_lsqr(tmp_path):
    import torch.multiprocessing as mp

    errfile = str(tmp_path / "err")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env_path = os.environ.get("PYTHONPATH", "")
    os.environ["PYTHONPATH"] = root + (os.pathsep + env_path if env_path else "")
    mp.spawn(_rank_main, args=(2, _free_port(), errfile), nprocs=2, join=True)
    for r in range(2):
        assert not os.path.exists(f"{errfile}.{r}"), open(f"{errfile}.{r}").read()
