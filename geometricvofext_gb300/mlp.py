"""Learned-normal network: tensor-core layers driven from Python.

The network maps an interface cell's neighbourhood (alpha and centroid
offsets / h of the cell and its 30 nearest stencil cells, plus their FP32
least-squares normal: 128 features) to a unit normal and a plane constant.
Four 128 x 128 layers with BF16 weights and activations, FP32 accumulation,
GELU between layers; outputs 0-2 correct the least-squares normal (the
normal is normalise(n_ls + y[0:3])), output 3 is the plane constant
(d + n.C) / h, outputs 4-127 are unused (their weights stay zero).

Every matrix product of training and inference runs in ``simplic_mlp_gemm``
(tcgen05.mma, csrc/mlp_kernels.cu); torch provides device memory and the
elementwise glue (the loss gradient of the four outputs and Adam).  Training
samples come from ``Simplic.samples`` (the step's own cut-cell volumes).
The product path fails if the CUDA library is missing.

    python -m geometricvofext_gb300.mlp --out normal_net.npz   # train on the GPU
"""

from __future__ import annotations

import argparse
import ctypes as C
import math
import os
import time

import numpy as np

from . import capi

STORE, ATOMIC, BIAS, BIAS_GELU, GELU_BACKWARD = 0, 1, 2, 3, 4
WIDTH = 128
N_LAYERS = 4
N_OUT = 4  # normal (3) + plane constant
D_WEIGHT = 0.1  # weight of the plane-constant term in the loss
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "normal_net.npz")


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def gemm(A, B, mode, D=None, bias=None, H=None, HT=None, Zin=None, split_k=1, err=None, stream=None):
    """D / H = A @ B.T with the epilogue ``mode`` (see include/simplic_mlp.h).
    A [M, K], B [N, K] BF16 contiguous torch CUDA tensors."""
    import torch

    M, K = A.shape
    N = B.shape[0]
    if err is None:
        err = torch.zeros(1, dtype=torch.int32, device=A.device)
    st = stream if stream is not None else torch.cuda.current_stream(A.device).cuda_stream
    r = capi.load().simplic_mlp_gemm(
        _p(A), A.stride(0), _p(B), B.stride(0), M, N, K, mode, _p(D), 0 if D is None else D.stride(0), _p(bias),
        _p(H), 0 if H is None else H.stride(0), _p(HT), 0 if HT is None else HT.stride(0), _p(Zin),
        0 if Zin is None else Zin.stride(0), split_k, _p(err), C.c_void_p(st))
    if r != 0:
        raise RuntimeError(f"simplic_mlp_gemm failed ({r})")
    return err


def init_params(seed=0):
    """He-style initial weights (FP32, host): W [4, 128, 128], b [4, 128];
    rows of the last layer beyond the outputs are zero."""
    rng = np.random.default_rng(seed)
    W = rng.normal(0.0, 1.0, (N_LAYERS, WIDTH, WIDTH)).astype(np.float32) * np.float32(math.sqrt(2.0 / WIDTH))
    W[-1, N_OUT:, :] = 0.0
    W[-1] *= 0.1
    b = np.zeros((N_LAYERS, WIDTH), np.float32)
    return W, b


LS_SLOT = 124  # features 124..126: the least-squares normal the network corrects


def normals_from_outputs(X, Y):
    """normalise(n_ls + y[0:3]): the network's normal from its input row and
    output (torch tensors)."""
    import torch

    n = X[:, LS_SLOT:LS_SLOT + 3].float() + Y[:, :3]
    return n / torch.clamp(n.norm(dim=1, keepdim=True), min=1e-6)


def loss_and_grad(Y, T, X):
    """Loss of the outputs Y[:, :4] (FP32) against targets T (normal, plane
    constant) and its gradient dL/dY (FP32, zero beyond the outputs)."""
    import torch

    y = Y[:, :N_OUT].detach().requires_grad_(True)
    nn = normals_from_outputs(X, y)
    cos = (nn * T[:, :3]).sum(1)
    L = (1.0 - cos).mean() + D_WEIGHT * ((y[:, 3] - T[:, 3]) ** 2).mean()
    (g,) = torch.autograd.grad(L, y)
    dY = torch.zeros_like(Y)
    dY[:, :N_OUT] = g
    return float(L.item()), dY


class Trainer:
    """Forward / backward of the network with the tensor-core GEMM; FP32
    master weights and Adam on the device."""

    def __init__(self, W, b, batch, device="cuda", lr=2e-3):
        import torch

        self.t = torch
        self.dev = torch.device(device)
        self.B = batch
        self.W = torch.tensor(W, device=self.dev)
        self.b = torch.tensor(b, device=self.dev)
        self.mW = torch.zeros_like(self.W)
        self.vW = torch.zeros_like(self.W)
        self.mb = torch.zeros_like(self.b)
        self.vb = torch.zeros_like(self.b)
        self.lr = lr
        self.step_no = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        f32, bf = torch.float32, torch.bfloat16
        B = batch
        self.Z = [torch.empty((B, WIDTH), dtype=f32, device=self.dev) for _ in range(N_LAYERS - 1)]
        self.H = [torch.empty((B, WIDTH), dtype=bf, device=self.dev) for _ in range(N_LAYERS - 1)]
        self.HT = [torch.empty((WIDTH, B), dtype=bf, device=self.dev) for _ in range(N_LAYERS - 1)]
        self.Y = torch.empty((B, WIDTH), dtype=f32, device=self.dev)
        self.dZ = torch.empty((B, WIDTH), dtype=bf, device=self.dev)
        self.dZT = torch.empty((WIDTH, B), dtype=bf, device=self.dev)
        self.dZ2 = torch.empty((B, WIDTH), dtype=bf, device=self.dev)
        self.dZ2T = torch.empty((WIDTH, B), dtype=bf, device=self.dev)
        self.gW = torch.zeros_like(self.W)
        self.gb = torch.zeros_like(self.b)
        self._refresh()

    def _refresh(self):
        self.Wb = self.W.to(self.t.bfloat16).contiguous()
        self.WbT = self.W.transpose(1, 2).to(self.t.bfloat16).contiguous()

    def forward(self, X):
        """X BF16 [B, 128] -> Y FP32 [B, 128] (keeps Z, H for backward)."""
        A = X
        for l in range(N_LAYERS - 1):
            gemm(A, self.Wb[l], BIAS_GELU, D=self.Z[l], bias=self.b[l], H=self.H[l], HT=self.HT[l], err=self.err)
            A = self.H[l]
        gemm(A, self.Wb[-1], BIAS, D=self.Y, bias=self.b[-1], err=self.err)
        return self.Y

    def backward(self, X, dY, split_k=8):
        """Gradients of all weights and biases for dL/dY (FP32 [B, 128])."""
        t = self.t
        XT = X.transpose(0, 1).contiguous()
        self.gW.zero_()
        dYb = dY.to(t.bfloat16)
        dYT = dYb.transpose(0, 1).contiguous()
        L = N_LAYERS - 1
        # output layer
        gemm(dYT, self.HT[L - 1], ATOMIC, D=self.gW[L], split_k=split_k, err=self.err)
        self.gb[L] = dY.sum(0)
        gemm(dYb, self.WbT[L], GELU_BACKWARD, H=self.dZ, HT=self.dZT, Zin=self.Z[L - 1], err=self.err)
        cur, curT, nxt, nxtT = self.dZ, self.dZT, self.dZ2, self.dZ2T
        for l in range(L - 1, -1, -1):
            inT = self.HT[l - 1] if l > 0 else XT
            gemm(curT, inT, ATOMIC, D=self.gW[l], split_k=split_k, err=self.err)
            self.gb[l] = cur.float().sum(0)
            if l > 0:
                gemm(cur, self.WbT[l], GELU_BACKWARD, H=nxt, HT=nxtT, Zin=self.Z[l - 1], err=self.err)
                cur, curT, nxt, nxtT = nxt, nxtT, cur, curT
        return self.gW, self.gb

    def adam(self, lr=None, b1=0.9, b2=0.999, eps=1e-8):
        lr = self.lr if lr is None else lr
        self.step_no += 1
        c1 = 1 - b1 ** self.step_no
        c2 = 1 - b2 ** self.step_no
        for p, g, m, v in ((self.W, self.gW, self.mW, self.vW), (self.b, self.gb, self.mb, self.vb)):
            m.mul_(b1).add_(g, alpha=1 - b1)
            v.mul_(b2).addcmul_(g, g, value=1 - b2)
            p.addcdiv_(m / c1, (v / c2).sqrt_().add_(eps), value=-lr)
        self.W[-1, N_OUT:, :] = 0.0
        self.b[-1, N_OUT:] = 0.0
        self._refresh()

    def weights(self):
        return self.W.cpu().numpy().copy(), self.b.cpu().numpy().copy()


def forward_fused(W, b, X, stream=None):
    """The step's inference kernel (all four layers in one tcgen05 kernel):
    FP32 outputs [n, 16] of the rows of X (BF16 [n, 128])."""
    import torch

    n = X.shape[0]
    Wb = torch.tensor(W, device=X.device).to(torch.bfloat16).contiguous()
    bt = torch.tensor(b, device=X.device).contiguous()
    Y = torch.empty((n, 16), dtype=torch.float32, device=X.device)
    M = torch.tensor([n], dtype=torch.int32, device=X.device)
    err = torch.zeros(1, dtype=torch.int32, device=X.device)
    st = stream if stream is not None else torch.cuda.current_stream(X.device).cuda_stream
    r = capi.load().simplic_mlp_forward(_p(X), _p(M), n, _p(Wb), _p(bt), _p(Y), 16, _p(err), C.c_void_p(st))
    if r != 0:
        raise RuntimeError(f"simplic_mlp_forward failed ({r})")
    return Y, err


def predict_normals(W, b, X):
    """Inference with the tensor-core GEMM: unit normals and plane constants
    of the rows of X (BF16 [n, 128], n a multiple of 128)."""
    tr = Trainer(W, b, X.shape[0])
    Y = tr.forward(X)
    return normals_from_outputs(X, Y), Y[:, 3]


def make_samples(meshes, count, seed, sphere_percent=50):
    """count samples spread over the given meshes (handles are created on
    the current device); returns X BF16 [count, 128], T FP32 [count, 4]."""
    import torch

    X = torch.empty((count, WIDTH), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((count, 4), dtype=torch.float32, device="cuda")
    per = count // len(meshes)
    off = 0
    for k, mesh in enumerate(meshes):
        n = per if k < len(meshes) - 1 else count - off
        g = capi.Simplic(mesh)
        g.samples(seed + 7919 * k, X[off:off + n], T[off:off + n], sphere_percent)
        g.synchronize()
        g.close()
        off += n
    return X, T


def train(samples=1 << 21, batch=8192, epochs=6, seed=1, lr=2e-3, log=print):
    """Train on seeded samples from a jittered hex mesh, a tet mesh and a
    uniform hex mesh; returns (W, b, history)."""
    import torch

    from . import meshgen as mg

    meshes = [mg.make_mesh("jitter", 32), mg.make_mesh("tet", 16), mg.make_mesh("hex", 32)]
    t0 = time.time()
    X, T = make_samples(meshes, samples, seed)
    torch.cuda.synchronize()
    log(f"samples: {samples} in {time.time() - t0:.1f} s")
    W, b = init_params(seed)
    tr = Trainer(W, b, batch, lr=lr)
    nb = samples // batch
    total = epochs * nb
    g = torch.Generator(device="cuda").manual_seed(seed)
    hist = []
    it = 0
    for ep in range(epochs):
        perm = torch.randperm(samples, device="cuda", generator=g)
        run = 0.0
        for k in range(nb):
            idx = perm[k * batch:(k + 1) * batch]
            Xb, Tb = X[idx].contiguous(), T[idx].contiguous()
            Y = tr.forward(Xb)
            L, dY = loss_and_grad(Y, Tb, Xb)
            tr.backward(Xb, dY)
            lr_k = lr * 0.5 * (1 + math.cos(math.pi * it / total))
            tr.adam(lr_k)
            run += L
            it += 1
        hist.append(run / nb)
        log(f"epoch {ep}: loss {run / nb:.5f} ({time.time() - t0:.1f} s)")
    if int(tr.err.item()) != 0:
        raise RuntimeError("tensor-core GEMM reported a device error")
    W, b = tr.weights()
    return W, b, hist


def save(path, W, b, **meta):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, W=W, b=b, **meta)


def load_weights(path=DEFAULT_WEIGHTS):
    d = np.load(path)
    return d["W"], d["b"]


def main():
    ap = argparse.ArgumentParser(description="train the learned-normal network on the GPU")
    ap.add_argument("--samples", type=int, default=1 << 21)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    W, b, hist = train(a.samples, a.batch, a.epochs, a.seed)
    save(a.out, W, b, loss=np.asarray(hist), samples=a.samples, epochs=a.epochs, seed=a.seed)
    print("saved", a.out)


if __name__ == "__main__":
    main()
