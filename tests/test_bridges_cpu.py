"""Preconditioned inversion and the torch bridge on host operators (dense
matrices), against the reference's own results (golden vectors) and torch
autograd."""

import numpy as np
import pytest

from tests.helpers import load, rel


def test_preconditioned_inversion_matches_reference_on_a_matrix():
    from pylops_gb300.basicoperators import Diagonal
    from pylops_gb300.linearoperator import aslinearoperator
    from pylops_gb300.optimization import PreconditionedInversion, preconditioned_inversion

    g = load("precond_inversion")
    Op = aslinearoperator(g["A"])
    P = Diagonal(g["pa"])
    xs, istop, itn, r1, r2 = preconditioned_inversion(Op, g["ya"], P, engine="scipy", iter_lim=30)
    assert itn == int(g["xa_scipy_iit"]) and rel(xs, g["xa_scipy"]) < 1e-10
    xp, istop, itn, r1, r2 = preconditioned_inversion(Op, g["ya"], P, engine="pylops", niter=12, tol=1e-12)
    assert itn == int(g["xa_pylops_iit"]) and rel(xp, g["xa_pylops"]) < 1e-10
    np.testing.assert_allclose(r1, float(g["xa_pylops_r1"]), rtol=1e-8)
    with pytest.raises(NotImplementedError):
        PreconditionedInversion(Op).step()
    with pytest.raises(NotImplementedError):
        preconditioned_inversion(Op, g["ya"], P, engine="other")


def test_torch_operator_forward_and_gradient():
    torch = pytest.importorskip("torch")
    from pylops_gb300 import TorchOperator
    from pylops_gb300.linearoperator import aslinearoperator

    rng = np.random.default_rng(0)
    A = rng.standard_normal((7, 5))
    Top = TorchOperator(aslinearoperator(A))
    x = torch.tensor(rng.standard_normal(5), requires_grad=True)
    w = torch.tensor(rng.standard_normal(7))
    y = Top(x)
    assert np.allclose(y.detach().numpy(), A @ x.detach().numpy())
    (y * w).sum().backward()
    assert np.allclose(x.grad.numpy(), A.T @ w.numpy())
    # batch of samples along the first axis
    Tb = TorchOperator(aslinearoperator(A), batch=True)
    X = torch.tensor(rng.standard_normal((3, 5)), requires_grad=True)
    Y = Tb(X)
    assert np.allclose(Y.detach().numpy(), X.detach().numpy() @ A.T)
    Y.sum().backward()
    assert np.allclose(X.grad.numpy(), np.ones((3, 7)) @ A)


def test_solver_callbacks_order_and_models():
    """Callbacks around setup/step/run: begin hooks in list order, end hooks
    in reverse order, setup sees the x0 keyword and step/run their first
    argument (basesolver.py:80-120), with one notification per call."""
    from pylops_gb300.linearoperator import aslinearoperator
    from pylops_gb300.optimization.callback import Callbacks
    from pylops_gb300.optimization.cls_basic import CGLS, LSQR

    log = []

    class Rec(Callbacks):
        def __init__(self, tag):
            self.tag = tag

        def on_setup_begin(self, solver, x0):
            log.append((self.tag, "setup_begin", None if x0 is None else x0.shape))

        def on_setup_end(self, solver, x):
            log.append((self.tag, "setup_end"))

        def on_step_begin(self, solver, x):
            log.append((self.tag, "step_begin", x.shape))

        def on_step_end(self, solver, x):
            log.append((self.tag, "step_end"))

        def on_run_begin(self, solver, x):
            log.append((self.tag, "run_begin"))

        def on_run_end(self, solver, x):
            log.append((self.tag, "run_end"))

    rng = np.random.default_rng(3)
    A = rng.standard_normal((9, 4))
    y = A @ rng.standard_normal(4)
    for cls in (CGLS, LSQR):
        log.clear()
        s = cls(aslinearoperator(A), callbacks=[Rec("a"), Rec("b")])
        x = s.setup(y, x0=np.zeros(4))
        x = s.run(x, niter=2)
        steps = [e for e in log if e[1].startswith("step")]
        assert log[:4] == [("a", "setup_begin", (4,)), ("b", "setup_begin", (4,)), ("b", "setup_end"),
                           ("a", "setup_end")], (cls, log[:4])
        assert log[4:6] == [("a", "run_begin"), ("b", "run_begin")]
        assert log[-2:] == [("b", "run_end"), ("a", "run_end")]
        assert steps == [("a", "step_begin", (4,)), ("b", "step_begin", (4,)), ("b", "step_end"),
                         ("a", "step_end")] * 2, (cls, steps)
