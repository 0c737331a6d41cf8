"""Failure detection of the library, with every fault made on the host.

The reference stops with FatalError on a bad orientation method or patch
(src/SimPLIC/reconstruction/reconstruction.C:610-625,
src/SimPLIC/advection/advectionTemplates.C:58-63) and otherwise carries bad
data along.  This library never aborts: each entry point returns a status
code with a message.  The cases:

* meshes the library cannot take (checked on the host before any device
  call, so these run without a GPU): a truncated face CSR, indices out of
  range, a cell with more faces or points than the static caps;
* a non-finite alpha, found by the mixed-cell scan;
* a device allocation that fails (the SIMPLIC_TEST_FAIL_ALLOC_AFTER test
  setting makes the n-th allocation of a create fail);
* a bounded device wait that runs out (the SIMPLIC_TEST_BARRIER_STALL test
  setting makes the bounding kernel's grid barrier wait for a block that
  never arrives; the wait gives up after the given number of polls and
  every block ends): the step reports the timeout and the library stays
  usable;
* resume: N steps equal k steps, the field saved to the host and loaded into
  a new handle, and N - k more steps, bit for bit.
"""

import ctypes as C
import os

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg
from oracle import oracle as O


def _desc(mesh, **override):
    arrs = {
        "points": np.ascontiguousarray(mesh.points, np.float64),
        "face_offsets": np.ascontiguousarray(mesh.face_offsets, np.int32),
        "face_points": np.ascontiguousarray(mesh.face_points, np.int32),
        "owner": np.ascontiguousarray(mesh.owner, np.int32),
        "neighbour": np.ascontiguousarray(mesh.neighbour, np.int32),
        "C": np.ascontiguousarray(mesh.C, np.float64),
        "V": np.ascontiguousarray(mesh.V, np.float64),
        "Cf": np.ascontiguousarray(mesh.Cf, np.float64),
        "Sf": np.ascontiguousarray(mesh.Sf, np.float64),
        "magSf": np.ascontiguousarray(mesh.magSf, np.float64),
    }
    arrs.update(override)
    d = capi.MeshDesc(int(arrs["points"].shape[0]), int(arrs["owner"].size), int(arrs["neighbour"].size),
                      int(override.get("n_cells", mesh.n_cells)),
                      *(arrs[k].ctypes.data_as(C.POINTER(C.c_double if arrs[k].dtype == np.float64 else C.c_int32))
                        for k in ("points", "face_offsets", "face_points", "owner", "neighbour", "C", "V", "Cf",
                                  "Sf", "magSf")))
    return d, arrs


def _create(desc):
    L = capi.load()
    h = C.c_void_p()
    r = L.simplic_create(C.byref(desc), None, None, C.byref(h))
    msg = L.simplic_last_error(None).decode()
    if r == 0:
        L.simplic_destroy(h)
    return r, msg


def test_truncated_face_csr_is_rejected():
    m = mg.hex_mesh(3)
    fo = m.face_offsets.copy()
    fo[-1] = fo[-2]  # the last face lost its points
    d, keep = _desc(m, face_offsets=fo)
    r, msg = _create(d)
    assert r == 1 and "fewer than 3 points" in msg
    fo = m.face_offsets.copy()
    fo[0] = 4
    d, keep = _desc(m, face_offsets=fo)
    r, msg = _create(d)
    assert r == 1 and "face_offsets[0]" in msg


def test_indices_out_of_range_are_rejected():
    m = mg.hex_mesh(3)
    fp = m.face_points.copy()
    fp[5] = m.n_points
    d, keep = _desc(m, face_points=fp)
    assert _create(d) == (1, "face point index out of range")
    ow = m.owner.copy()
    ow[-1] = -1
    d, keep = _desc(m, owner=ow)
    assert _create(d) == (1, "owner out of range")
    nb = m.neighbour.copy()
    nb[0] = m.owner[0]
    d, keep = _desc(m, neighbour=nb)
    assert _create(d) == (1, "neighbour out of range")


def _split_cube_cell(k):
    """One unit-cube cell whose bottom face is split into k x k quads:
    5 + k^2 faces and 4 + (k + 1)^2 points, all boundary faces."""
    pts = [(i / k, j / k, 0.0) for j in range(k + 1) for i in range(k + 1)]
    top = len(pts)
    pts += [(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    pid = lambda i, j: i + (k + 1) * j  # noqa: E731
    faces = []
    for j in range(k):
        for i in range(k):  # normals -z (out of the cell)
            faces.append([pid(i, j), pid(i, j + 1), pid(i + 1, j + 1), pid(i + 1, j)])
    faces.append([top, top + 1, top + 2, top + 3])  # +z
    faces.append([pid(0, 0), pid(k, 0), top + 1, top])  # -y
    faces.append([pid(k, 0), pid(k, k), top + 2, top + 1])  # +x
    faces.append([pid(k, k), pid(0, k), top + 3, top + 2])  # +y
    faces.append([pid(0, k), pid(0, 0), top, top + 3])  # -x
    return np.array(pts, np.float64), faces


def _poly_mesh(pts, faces, n_cells=1):
    nf = len(faces)
    off = np.concatenate(([0], np.cumsum([len(f) for f in faces]))).astype(np.int32)
    P = np.asarray(pts)
    Cf = np.array([P[f].mean(axis=0) for f in faces])
    Sf = np.zeros((nf, 3))
    for q, f in enumerate(faces):
        for i in range(len(f)):
            a, b = P[f[i]], P[f[(i + 1) % len(f)]]
            Sf[q] += 0.5 * np.cross(a - Cf[q], b - Cf[q])
    m = mg.PolyMesh(points=P, face_offsets=off, face_points=np.concatenate(faces).astype(np.int32),
                    owner=np.zeros(nf, np.int32), neighbour=np.zeros(0, np.int32), n_cells=n_cells,
                    patches=[("walls", 0, nf)])
    m.Cf, m.Sf, m.magSf = Cf, Sf, np.linalg.norm(Sf, axis=1)
    m.C = np.array([[0.5, 0.5, 0.5]])
    m.V = np.array([1.0])
    return m


def test_cell_over_the_static_caps_is_rejected():
    pts, faces = _split_cube_cell(7)  # 54 faces, 68 points
    d, keep = _desc(_poly_mesh(pts, faces))
    r, msg = _create(d)
    assert r == 3, msg  # SIMPLIC_ERR_MESH_CAPS
    assert "exceeds" in msg


# ---------------------------------------------------------------------------
# on the GPU
# ---------------------------------------------------------------------------

def _case(n=16, cfl=1.0):
    m = mg.hex_mesh(n)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = cfl * H.cfl_delta_t(m, flow.phi0)
    return m, a0, flow, dt


@pytest.mark.gpu
def test_non_finite_alpha_is_reported():
    m, a0, flow, dt = _case()
    g = capi.Simplic(m)
    for bad in (np.nan, np.inf, -np.inf):
        a = a0.copy()
        a[123] = bad
        with pytest.raises(capi.SimplicError) as e:
            g.reconstruct(a)
        assert e.value.code == 4 and "non-finite-alpha" in str(e.value)
    # the handle keeps working on a clean field
    g.reconstruct(a0)
    assert g.stats()[0] > 0


@pytest.mark.gpu
def test_device_allocation_failure_is_reported(monkeypatch):
    m, a0, flow, dt = _case(8)
    for n in (0, 3, 12, 30, 45):
        monkeypatch.setenv("SIMPLIC_TEST_FAIL_ALLOC_AFTER", str(n))
        with pytest.raises(capi.SimplicError) as e:
            capi.Simplic(m)
        assert e.value.code == 2 and "cudaMalloc failed" in str(e.value)
    monkeypatch.delenv("SIMPLIC_TEST_FAIL_ALLOC_AFTER")
    g = capi.Simplic(m)
    g.reconstruct(a0)
    assert g.stats()[0] > 0


@pytest.mark.gpu
def test_bounding_barrier_timeout_is_reported_and_the_library_recovers(monkeypatch):
    """Twice the Courant-0.5 step makes cells overshoot, so the bounding
    kernel runs and meets its first grid barrier, which here waits for one
    block more than the grid has: every block gives up after 20000 polls
    and ends.  The step returns SIMPLIC_ERR_DEVICE with the timeout; a
    handle made without the setting then steps bit for bit with the
    oracle, bounding included."""
    m, a0, flow, dt = _case(16, cfl=2.0)
    monkeypatch.setenv("SIMPLIC_TEST_BARRIER_STALL", "20000")
    g = capi.Simplic(m, n_alpha_bounds=3, clip=0)
    monkeypatch.delenv("SIMPLIC_TEST_BARRIER_STALL")
    a = a0.copy()
    err = None
    for s in range(6):
        fl = flow.at((s + 1) * dt, dt)
        g.reconstruct(a)
        try:
            a = g.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        except capi.SimplicError as e:
            err = e
            break
    assert err is not None and err.code == 4 and "grid-barrier-timeout" in str(err)
    g.close()
    g = capi.Simplic(m, n_alpha_bounds=3, clip=0)
    o = O.Oracle(m, n_alpha_bounds=3, clip=False)
    ag, ao = a0.copy(), a0.copy()
    bounded = 0
    for s in range(6):
        fl = flow.at((s + 1) * dt, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        np.testing.assert_array_equal(ag, ao)
        bounded = max(bounded, g.stats()[2])
    assert bounded > 0  # the bounding really ran


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [capi.PRECISION_PLAIN_FP64, capi.PRECISION_MIXED])
def test_resume_is_bit_exact(precision):
    """The advection state is alpha (the reconstruction is recomputed every
    step): 12 steps in one handle equal 5 steps, alpha saved to the host,
    a new handle loaded with it, and 7 more steps, bit for bit; through the
    device-resident entry points."""
    torch = pytest.importorskip("torch")
    m, a0, flow, dt = _case(20)
    dev = torch.device("cuda", 0)
    steps, k = 12, 5

    def run(g, first, last):
        for s in range(first, last):
            fl = flow.at((s + 1) * dt, dt)
            phi = torch.from_numpy(fl.phi).to(dev)
            U = torch.from_numpy(fl.U).to(dev)
            Ub = torch.from_numpy(fl.U_boundary).to(dev)
            torch.cuda.synchronize()
            g.reconstruct_resident()
            g.advect_resident(phi, U, dt, U_boundary=Ub)
            g.synchronize()

    g = capi.Simplic(m, precision=precision, n_alpha_bounds=3, clip=0)
    g.set_alpha(a0)
    run(g, 0, steps)
    whole = g.get_alpha()
    g1 = capi.Simplic(m, precision=precision, n_alpha_bounds=3, clip=0)
    g1.set_alpha(a0)
    run(g1, 0, k)
    saved = g1.get_alpha()
    g1.close()
    g2 = capi.Simplic(m, precision=precision, n_alpha_bounds=3, clip=0)
    g2.set_alpha(saved)
    run(g2, k, steps)
    np.testing.assert_array_equal(g2.get_alpha(), whole)
