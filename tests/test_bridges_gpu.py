"""Preconditioned inversion of a Kirchhoff operator (device CGLS on K diag(p))
against the reference's result, and the torch bridge on CUDA tensors."""

import numpy as np
import pytest

from tests.helpers import kwargs_from_golden, load, rel

pytestmark = pytest.mark.gpu


def _op():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = kwargs_from_golden(load("k2d_dyn_noap"))
    return Kirchhoff(*args, engine="cuda", dtype="float32", **kw)


def test_preconditioned_inversion_of_kirchhoff_matches_reference():
    import torch

    from pylops_gb300.basicoperators import Diagonal
    from pylops_gb300.optimization import preconditioned_inversion
    from pylops_gb300.optimization.cls_basic import _is_device_kirchhoff

    g = load("precond_inversion")
    K = _op()
    P = Diagonal(g["p"].astype(np.float32), dtype="float32")
    assert _is_device_kirchhoff(K @ P)
    d = torch.as_tensor(g["d"].astype(np.float32), device="cuda")
    x, istop, itn, r1, r2 = preconditioned_inversion(K, d, P, engine="pylops", niter=8, tol=1e-10)
    assert x.is_cuda and itn == int(g["xk_iit"])
    assert rel(x.cpu().numpy(), g["xk"]) < 1e-4
    np.testing.assert_allclose(r1, float(g["xk_r1"]), rtol=1e-3)


def test_torch_operator_on_cuda_tensors():
    import torch

    from pylops_gb300 import TorchOperator

    K = _op()
    Top = TorchOperator(K, device="gpu", devicetorch="cuda")
    x = torch.randn(K.shape[1], device="cuda", requires_grad=True)
    y = Top(x)
    assert y.is_cuda and torch.allclose(y, K @ x.detach(), rtol=0, atol=0)
    w = torch.randn(K.shape[0], device="cuda")
    (y * w).sum().backward()
    assert torch.allclose(x.grad, K.H @ w, rtol=0, atol=0)
