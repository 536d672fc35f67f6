"""The tcgen05 BF16 GEMM against a float32 torch reference of the same op
(bf16 inputs are exact in float32; float32 accumulation in both)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(A, B, bias=None, flags=0, out_bf16=False):
    import torch

    from pylops_gb300 import _native

    M, K = A.shape
    N = B.shape[0]
    C = torch.empty(M, N, dtype=torch.bfloat16 if out_bf16 else torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _native.check(_native.lib().kgb_gemm_bf16_tn(
        A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, A.stride(0), B.stride(0), C.stride(0),
        0 if bias is None else bias.data_ptr(), flags | (2 if out_bf16 else 0), err.data_ptr(),
        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return C


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 256), (300, 96, 72), (130, 32, 16), (1000, 256, 520)])
def test_gemm_matches_fp32_reference(M, N, K):
    import torch

    g = torch.Generator(device="cpu").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    ref = A.float() @ B.float().T
    C = _gemm(A, B)
    err = (C - ref).norm() / ref.norm()
    assert err < 1e-5, float(err)


def test_gemm_bias_relu_and_bf16_output():
    import torch

    g = torch.Generator(device="cpu").manual_seed(5)
    A = torch.randn(200, 40, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(48, 40, generator=g).to(torch.bfloat16).cuda()
    bias = torch.randn(48, generator=g).cuda()
    ref = torch.relu(A.float() @ B.float().T + bias)
    C = _gemm(A, B, bias=bias, flags=1)
    assert ((C - ref).norm() / ref.norm()) < 1e-5
    Cb = _gemm(A, B, bias=bias, flags=1, out_bf16=True)
    assert ((Cb.float() - ref).norm() / ref.norm()) < 1e-2
