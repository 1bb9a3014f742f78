"""Learned preconditioner kernels: the tcgen05 BF16 GEMM against an FP64 product of the same
bf16 operands."""

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from stride_gb300 import _lib  # noqa: E402

pytestmark = pytest.mark.gpu


def _gemm(A, B, C=None, bias=None, relu=False, accumulate=False, want_bf16=False):
    M, K = A.shape
    N = B.shape[0]
    C = torch.zeros((M, N), device='cuda') if C is None else C
    Cb = torch.zeros((M, N), dtype=torch.bfloat16, device='cuda') if want_bf16 else None
    err = torch.zeros(1, dtype=torch.int32, device='cuda')
    _lib.check(_lib.load().sa_gemm_bf16(_lib._ptr(A), A.stride(0), _lib._ptr(B), B.stride(0), _lib._ptr(C), C.stride(0),
                                        _lib._ptr(Cb), N, M, N, K, _lib._ptr(bias), int(relu), int(accumulate),
                                        _lib._ptr(err), _lib._stream(torch.cuda.current_stream())))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return C, Cb


@pytest.mark.parametrize('M,N,K', [(128, 32, 64), (256, 64, 128), (384, 128, 192), (128, 256, 64), (256, 96, 320)])
def test_gemm_bf16(M, N, K):
    g = torch.Generator(device='cpu').manual_seed(M + N + K)
    A = torch.randn((M, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((N, K), generator=g).to(torch.bfloat16).cuda()
    C, _ = _gemm(A, B)
    ref = A.double() @ B.double().T
    err = float((C.double() - ref).norm() / ref.norm())
    assert err <= 1e-5, err


def test_gemm_epilogue():
    g = torch.Generator(device='cpu').manual_seed(7)
    M, N, K = 256, 64, 128
    A = torch.randn((M, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((N, K), generator=g).to(torch.bfloat16).cuda()
    C0 = torch.randn((M, N), generator=g).cuda()
    bias = torch.randn(N, generator=g).cuda()
    C, Cb = _gemm(A, B, C=C0.clone(), bias=bias, relu=True, accumulate=True, want_bf16=True)
    ref = torch.relu(C0.double() + A.double() @ B.double().T + bias.double())
    assert float((C.double() - ref).norm() / ref.norm()) <= 1e-5
    assert torch.equal(Cb, C.to(torch.bfloat16))
