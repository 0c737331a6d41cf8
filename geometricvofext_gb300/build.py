"""Builds the CUDA library ``libsimplic_cuda.so`` in-tree for sm_103a.

Plain nvcc invocations, one object per translation unit compiled in
parallel, then one shared-library link.  The plain FP64 kernels are compiled
with ``-fmad=false`` (no fused multiply-add contraction) so they reproduce
the FP64 restatement bit for bit; host code uses ``-ffp-contract=off`` for
the same reason.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libsimplic_cuda.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include")]

# translation unit -> extra flags
UNITS = {
    "plain_kernels.cu": ["-fmad=false"],
    "plain_bound.cu": ["-fmad=false"],
    "rdf_kernels.cu": ["-fmad=false"],
    "plic_kernels.cu": ["-fmad=false"],
    "simplic_capi.cu": ["-fmad=false"],
    "noalloc_scan.cu": [],
    # mixed-precision form: fused multiply-add allowed
    "mixed_kernels.cu": [],
    # tensor-core layers of the learned-normal network, its inputs and samples
    "mlp_kernels.cu": [],
    "learned_kernels.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsimplic_cuda.so")


def _sources_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(ROOT, "include", "simplic.h"))
    paths.append(os.path.join(ROOT, "include", "simplic_mlp.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def up_to_date() -> bool:
    return os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _sources_mtime()


def _compile(unit: str, extra, verbose: bool):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_DIR, unit + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, f, verbose) for u, f in UNITS.items()]
        results = [f.result() for f in futs]
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
