"""tcgen05 GEMM of the learned-normal network against a plain PyTorch FP32
reference of the same operation (BF16 inputs, FP32 accumulation)."""

import pytest

torch = pytest.importorskip("torch")

from geometricvofext_gb300 import mlp  # noqa: E402

pytestmark = pytest.mark.gpu


def _bf(*shape, scale=1.0, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return (torch.randn(*shape, generator=g, device="cuda") * scale).to(torch.bfloat16)


def _gelu(z):
    return 0.5 * z * (1 + torch.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))


def _gelu_grad(z):
    u = 0.7978845608028654 * (z + 0.044715 * z ** 3)
    t = torch.tanh(u)
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * 0.7978845608028654 * (1 + 3 * 0.044715 * z * z)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 128, 128), (1000, 16, 128), (256, 256, 192)])
def test_gemm_store_matches_fp32(M, N, K):
    A, B = _bf(M, K, seed=1), _bf(N, K, seed=2)
    D = torch.full((M, N), float("nan"), device="cuda")
    err = mlp.gemm(A, B, mlp.STORE, D=D)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = A.float() @ B.float().T
    torch.testing.assert_close(D, ref, rtol=1e-4, atol=1e-4)


def test_gemm_split_k_atomic():
    M, N, K = 256, 128, 1024
    A, B = _bf(M, K, seed=3), _bf(N, K, seed=4)
    D = torch.zeros((M, N), device="cuda")
    mlp.gemm(A, B, mlp.ATOMIC, D=D, split_k=4)
    mlp.gemm(A, B, mlp.ATOMIC, D=D, split_k=3)  # accumulates
    torch.cuda.synchronize()
    torch.testing.assert_close(D, 2 * (A.float() @ B.float().T), rtol=1e-4, atol=1e-3)


def test_gemm_bias_gelu_and_transpose():
    M, N, K = 384, 128, 128
    A, B = _bf(M, K, scale=0.2, seed=5), _bf(N, K, scale=0.2, seed=6)
    bias = torch.linspace(-1, 1, N, device="cuda")
    Z = torch.zeros((M, N), device="cuda")
    H = torch.zeros((M, N), dtype=torch.bfloat16, device="cuda")
    HT = torch.zeros((N, M), dtype=torch.bfloat16, device="cuda")
    mlp.gemm(A, B, mlp.BIAS_GELU, D=Z, bias=bias, H=H, HT=HT)
    torch.cuda.synchronize()
    zref = A.float() @ B.float().T + bias
    torch.testing.assert_close(Z, zref, rtol=1e-4, atol=1e-4)
    torch.testing.assert_close(H.float(), _gelu(zref), rtol=1e-2, atol=1e-2)
    assert torch.equal(HT, H.T.contiguous())


def test_gemm_gelu_backward():
    M, N, K = 256, 128, 128
    A, B = _bf(M, K, scale=0.2, seed=7), _bf(N, K, scale=0.2, seed=8)
    Zin = torch.randn((M, N), device="cuda")
    H = torch.zeros((M, N), dtype=torch.bfloat16, device="cuda")
    mlp.gemm(A, B, mlp.GELU_BACKWARD, H=H, Zin=Zin)
    torch.cuda.synchronize()
    ref = (A.float() @ B.float().T) * _gelu_grad(Zin)
    torch.testing.assert_close(H.float(), ref, rtol=1e-2, atol=1e-2)
