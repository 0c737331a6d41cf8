"""CPU oracle of the learned-normal network (test infrastructure only).

Restates, in numpy, the forward and backward passes that
geometricvofext_gb300/mlp.py runs with the tensor-core GEMM, with the same
BF16 rounding points (weights, activations, backward deltas are BF16; sums
are carried in float64 here, FP32 on the GPU).  Only tests/ import this
module, to check the GPU gradients; the product never calls it.
"""

from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    u = 0.7978845608028654 * (z + 0.044715 * z ** 3)
    t = np.tanh(u)
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * 0.7978845608028654 * (1 + 3 * 0.044715 * z * z)


def forward(W, b, X):
    """W [L, 128, 128], b [L, 128] float32; X [n, 128] (BF16 values).
    Returns (Y, Z list, H list) with H BF16-rounded as on the GPU."""
    Wb = bf16(W).astype(np.float64)
    A = np.asarray(X, dtype=np.float64)
    Zs, Hs = [], []
    for l in range(W.shape[0] - 1):
        Z = A @ Wb[l].T + b[l]
        H = bf16(gelu(Z)).astype(np.float64)
        Zs.append(Z)
        Hs.append(H)
        A = H
    Y = A @ Wb[-1].T + b[-1]
    return Y, Zs, Hs


def backward(W, b, X, Zs, Hs, dY):
    """Gradients (gW, gb) of the weights for dL/dY, BF16 rounding of dY and
    of every delta as on the GPU."""
    Wb = bf16(W).astype(np.float64)
    L = W.shape[0] - 1
    gW = np.zeros(W.shape, np.float64)
    gb = np.zeros(b.shape, np.float64)
    dYb = bf16(dY).astype(np.float64)
    gW[L] = dYb.T @ Hs[L - 1]
    gb[L] = dY.sum(0)
    cur = bf16((dYb @ Wb[L]) * gelu_grad(Zs[L - 1])).astype(np.float64)
    for l in range(L - 1, -1, -1):
        inp = Hs[l - 1] if l > 0 else np.asarray(X, dtype=np.float64)
        gW[l] = cur.T @ inp
        gb[l] = cur.sum(0)
        if l > 0:
            cur = bf16((cur @ Wb[l]) * gelu_grad(Zs[l - 1])).astype(np.float64)
    return gW, gb
