"""Host-side checks that need no GPU: the C ABI library loads and exports
every entry point include/simplic.h declares, errors are reported (never
aborts), the fvSolution controls map like the reference's lookups, and the
replica timing reduction works across processes (gloo)."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from geometricvofext_gb300 import capi, meshgen as mg, replicas, solve_vof_equ as sve

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
            names |= set(re.findall(r"\b(simplic_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = capi.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(L, n), n
    assert set(capi.EXPORTS) <= names


def test_default_controls_match_reference_defaults():
    c = capi.default_controls()
    assert c.mixed_cell_tol == 1e-8 and c.n_alpha_bounds == 10 and c.snap_tol == 0.0 and c.clip == 1
    assert c.orientation_method == capi.ORIENTATION_ISO_ALPHA_GRAD and c.split_warped_face == 0


def _no_gpu():
    try:
        import torch

        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.mark.skipif(not _no_gpu(), reason="checks the no-device error path")
def test_create_without_device_reports_error():
    m = mg.hex_mesh(2)
    with pytest.raises(capi.SimplicError) as e:
        capi.Simplic(m)
    assert "CUDA" in str(e.value) or "device" in str(e.value)


def test_create_rejects_bad_arguments():
    L = capi.load()
    h = C.c_void_p()
    r = L.simplic_create(None, None, None, C.byref(h))
    assert r == 1 and not h.value
    assert b"mesh" in L.simplic_last_error(None)
    assert L.simplic_reconstruct(None, None) != 0


FV_SOLUTION = """
solvers
{
    "alpha.*"
    {
        nAlphaBounds        3;
        snapTol             0;
        clip                false;
        mixedCellTol        1e-8;
        orientationMethod   LS;    // least squares
        splitWarpedFace     false;
        nAlphaSubCycles     1;
    }
    p_rgh { solver PCG; tolerance 1e-7; }
}
PIMPLE { }
"""


def test_solver_dict_lookup_and_controls():
    d = sve.solver_dict(FV_SOLUTION, "alpha.water")
    assert d["nAlphaBounds"] == 3 and d["clip"] is False and d["orientationMethod"] == "LS"
    c = sve.controls_from_dict(d)
    assert c.n_alpha_bounds == 3 and c.clip == 0 and c.snap_tol == 0.0
    assert c.orientation_method == capi.ORIENTATION_ISO_ALPHA_GRAD
    c = sve.controls_from_dict({})
    assert c.n_alpha_bounds == 10 and c.clip == 1 and c.mixed_cell_tol == 1e-8
    with pytest.raises(ValueError):
        sve.controls_from_dict({"orientationMethod": "smoothAlphaGrad"})
    with pytest.raises(KeyError):
        sve.solver_dict(FV_SOLUTION, "T")
    # the form of the step: plain (default), mixed, learned; anything else is an error
    assert c.precision == capi.PRECISION_PLAIN_FP64
    for word, form in (("mixed", capi.PRECISION_MIXED), ("learned", capi.PRECISION_LEARNED)):
        assert sve.controls_from_dict({"precision": word}).precision == form
    with pytest.raises(ValueError):
        sve.controls_from_dict({"precision": "fp16"})


def test_replica_throughput():
    assert replicas.replica_throughput(2, 1000, 10, 100.0) == 2 * 1000 * 10 / 0.1
    with pytest.raises(ValueError):
        replicas.replica_throughput(1, 1, 1, 0.0)


def _gloo_worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    v = replicas.max_over_ranks(10.0 + 5.0 * rank, dist)
    out[rank] = v
    dist.destroy_process_group()


def test_max_over_ranks_gloo_two_processes():
    import torch.multiprocessing as mp

    port = 29500 + (os.getpid() % 2000)
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_gloo_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == 15.0 and out[1] == 15.0
