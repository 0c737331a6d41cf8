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


def test_network_gradients_match_cpu_oracle():
    """Forward and backward of the four tensor-core layers against the numpy
    oracle with the same BF16 rounding points."""
    np = pytest.importorskip("numpy")
    from oracle import mlp_oracle as MO

    rng = np.random.default_rng(3)
    W, b = mlp.init_params(5)
    W = W + rng.normal(0, 0.02, W.shape).astype(np.float32)
    W[-1, mlp.N_OUT:] = 0.0
    b = rng.normal(0, 0.1, b.shape).astype(np.float32)
    n = 256
    X = torch.tensor(MO.bf16(rng.normal(0, 1, (n, 128))), device="cuda").to(torch.bfloat16)
    dY = torch.zeros((n, 128), device="cuda")
    dY[:, :4] = torch.tensor(rng.normal(0, 1e-2, (n, 4)), dtype=torch.float32, device="cuda")
    tr = mlp.Trainer(W, b, n)
    Y = tr.forward(X).clone()
    gW, gb = tr.backward(X, dY, split_k=2)
    torch.cuda.synchronize()
    assert int(tr.err.item()) == 0
    Xh = X.float().cpu().numpy()
    Yo, Zs, Hs = MO.forward(W, b, Xh)
    gWo, gbo = MO.backward(W, b, Xh, Zs, Hs, dY.cpu().numpy())
    Yg = Y.cpu().numpy()
    assert np.linalg.norm(Yg[:, :4] - Yo[:, :4]) <= 1e-2 * np.linalg.norm(Yo[:, :4])
    for l in range(mlp.N_LAYERS):
        a, o = gW[l].cpu().numpy(), gWo[l]
        assert np.linalg.norm(a - o) <= 2e-2 * np.linalg.norm(o) + 1e-9, l
        a, o = gb[l].cpu().numpy(), gbo[l]
        assert np.linalg.norm(a - o) <= 2e-2 * np.linalg.norm(o) + 1e-9, l


def test_plane_samples_are_exact_volume_fractions():
    """Plane samples: unit normal labels, a cut centre cell, and features
    whose least-squares normal points along the label."""
    np = pytest.importorskip("numpy")
    from geometricvofext_gb300 import capi, meshgen as mg

    mesh = mg.make_mesh("hex", 16)
    g = capi.Simplic(mesh)
    n = 2048
    X = torch.empty((n, 128), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    g.samples(11, X, T, sphere_percent=0)
    g.synchronize()
    Xh = X.float().cpu().numpy().reshape(n, 32, 4)
    Th = T.cpu().numpy()
    assert np.allclose(np.linalg.norm(Th[:, :3], axis=1), 1.0, atol=1e-5)
    a0 = Xh[:, 0, 0]  # BF16: values within 1e-3 of 0 or 1 round onto them
    assert np.all((a0 >= 0) & (a0 <= 1)) and np.mean((a0 > 0) & (a0 < 1)) > 0.95
    # slot 31: the FP32 least-squares normal of the features, close to the
    # label for an exact plane
    ls = Xh[:, 31, :3]
    cosang = (ls * Th[:, :3]).sum(1) / np.maximum(np.linalg.norm(ls, axis=1), 1e-30)
    assert np.median(np.degrees(np.arccos(np.clip(cosang, -1, 1)))) < 10.0


def test_fused_network_matches_layer_by_layer():
    """The step's one-kernel network (weights and activations in shared
    memory) against the layer-by-layer tensor-core GEMMs of training."""
    np = pytest.importorskip("numpy")
    W, b = mlp.init_params(9)
    rng = np.random.default_rng(4)
    b = rng.normal(0, 0.1, b.shape).astype(np.float32)
    n = 1000  # not a multiple of 128
    X = torch.randn((1024, 128), device="cuda").to(torch.bfloat16)[:n].contiguous()
    Xp = torch.zeros((1024, 128), dtype=torch.bfloat16, device="cuda")
    Xp[:n] = X
    tr = mlp.Trainer(W, b, 1024)
    Yl = tr.forward(Xp)[:n, :16].clone()
    Yf, err = mlp.forward_fused(W, b, X)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    torch.testing.assert_close(Yf, Yl, rtol=1e-3, atol=1e-4)
