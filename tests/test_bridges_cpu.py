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
