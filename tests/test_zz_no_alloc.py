"""simplic_mixed_cells_noalloc against the handle's mixed-cell list.

The no-allocation entry point serves callers that may not call cudaMalloc
where they need the interface cells (their device memory belongs to their
own pool or framework allocator, or a fixed budget), so it works from plain
device pointers and a fixed scratch array inside the library.  Here the
caller's buffers come from torch; the check is that two calls in a row give
exactly the list that simplic_reconstruct + simplic_get_mixed_cells give for
the same alpha (an integer list: equality, no tolerance), including after
the scratch holds the previous call's contents.

This file is named to be collected last.
"""

import ctypes as C

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg

MAX_CELLS = 134217728
TOL = 1e-8


def _fn():
    L = capi.load()
    f = L.simplic_mixed_cells_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    return L, f


def test_noalloc_rejects_oversized_input():
    # rejected before any device work, so this runs without a GPU
    L, f = _fn()
    n = C.c_int32(-7)
    rc = f(None, MAX_CELLS + 1, TOL, None, 0, C.cast(C.pointer(n), C.c_void_p), None)
    assert rc == 1
    msg = L.simplic_last_error(None).decode()
    assert "134217728" in msg and "exceeds" in msg
    assert n.value == -7


@pytest.mark.gpu
def test_noalloc_matches_reconstruct_two_calls():
    import torch

    _, f = _fn()
    mesh = mg.make_mesh("hex", 24)
    flow = H.DeformationFlow(mesh)
    g = capi.Simplic(mesh, mixed_cell_tol=TOL)
    nc = mesh.n_cells

    a1 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    dt = 0.01
    fl = flow.at(dt, dt)
    g.reconstruct(a1)
    a2 = g.advect(a1, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
    # a second field with a different mixed-cell count (the list must come
    # from this call's counts alone)
    a3 = H.sphere_alpha(mesh, (0.5, 0.5, 0.5), 0.06)

    cells = torch.full((nc,), -1, dtype=torch.int32, device="cuda")
    n_dev = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    seen = []
    for a in (a2, a3):
        g.reconstruct(a)
        want, _ = g.mixed()
        a_dev = torch.from_numpy(np.ascontiguousarray(a)).to("cuda")
        cells.fill_(-1)
        rc = f(a_dev.data_ptr(), nc, TOL, cells.data_ptr(), nc, n_dev.data_ptr(), stream)
        assert rc == 0, capi.load().simplic_last_error(None)
        torch.cuda.synchronize()
        n = int(n_dev.item())
        got = cells.cpu().numpy()
        assert n == len(want)
        np.testing.assert_array_equal(got[:n], want)
        assert np.all(got[n:] == -1)
        seen.append(n)
    assert seen[0] > 0 and seen[1] > 0 and seen[1] != seen[0]

    # a short output buffer: the full count, only `capacity` cells written
    cap = seen[1] // 2
    cells.fill_(-1)
    rc = f(a_dev.data_ptr(), nc, TOL, cells.data_ptr(), cap, n_dev.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize()
    got = cells.cpu().numpy()
    assert int(n_dev.item()) == seen[1]
    np.testing.assert_array_equal(got[:cap], want[:cap])
    assert np.all(got[cap:] == -1)


@pytest.mark.gpu
def test_noalloc_many_tiles_edge_values():
    """5,000,001 cells (2442 tiles of 2048, the last one partial), so the
    one-block tile scan gives every thread several tiles and carries run
    offsets between them.  The alpha values include the exact bounds tol and
    1 - tol, -0.0, +0.0, NaN of both signs, infinities, denormals and values
    one ulp inside the bounds; the list must equal the ascending cells with
    tol < alpha < 1 - tol, on two calls in a row."""
    import torch

    _, f = _fn()
    n = 5_000_001
    rng = np.random.default_rng(7)
    a = rng.uniform(-0.2, 1.2, n)
    edge = np.array([TOL, 1.0 - TOL, -0.0, 0.0, np.nan, -np.nan, np.inf, -np.inf, 5e-324, -5e-324,
                     np.nextafter(TOL, 1.0), np.nextafter(1.0 - TOL, 0.0), np.nextafter(TOL, 0.0),
                     np.nextafter(1.0 - TOL, 2.0), 0.5, 1.0])
    pos = rng.choice(n, size=4000, replace=False)
    a[pos] = edge[np.arange(pos.size) % edge.size]
    a[-edge.size:] = edge  # the partial last tile holds them too
    with np.errstate(invalid="ignore"):
        want = np.flatnonzero((a > TOL) & (a < 1.0 - TOL)).astype(np.int32)
    a_dev = torch.from_numpy(a).to("cuda")
    cells = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    n_dev = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        cells.fill_(-1)
        rc = f(a_dev.data_ptr(), n, TOL, cells.data_ptr(), n, n_dev.data_ptr(), stream)
        assert rc == 0, capi.load().simplic_last_error(None)
        torch.cuda.synchronize()
        assert int(n_dev.item()) == want.size
        got = cells.cpu().numpy()
        np.testing.assert_array_equal(got[:want.size], want)
        assert np.all(got[want.size:] == -1)
