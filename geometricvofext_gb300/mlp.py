"""Learned-normal network: tensor-core layers driven from Python.

The network maps an interface cell's neighbourhood (alpha and centroid
offsets / h of up to 32 cells: 128 features) to a unit normal and a plane
constant.  Four 128 x 128 BF16 layers, FP32 accumulation, GELU between
layers; outputs 0-2 are the normal (normalised afterwards), output 3 the
plane constant in units of h relative to the cell centre.

Every matrix product runs in ``simplic_mlp_gemm`` (tcgen05.mma, see
csrc/mlp_kernels.cu); torch provides device memory and the elementwise glue
of the optimiser.  The product path fails if the CUDA library is missing.
"""

from __future__ import annotations

import ctypes as C

from . import capi

STORE, ATOMIC, BIAS, BIAS_GELU, GELU_BACKWARD = 0, 1, 2, 3, 4
WIDTH = 128
N_LAYERS = 4
N_OUT = 4  # normal (3) + plane constant


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
