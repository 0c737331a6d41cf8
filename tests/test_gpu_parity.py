"""CUDA path vs the CPU oracle, through the C ABI.

The plain form is FP64 and bit-exact by construction (same operation order,
no fused multiply-add on either side), so every comparison here asserts
exact equality.  The tolerance the target states -- alpha within 1e-10
absolute, classification identical, volume drift <= 1e-12 relative -- is
checked as well so a failure message shows which bar broke.
"""

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ALPHA_TOL = 1e-10


def _mesh(kind, n):
    return mg.make_mesh(kind, n)


def _pair(mesh, **kw):
    okw = dict(mixed_cell_tol=kw.get("mixed_cell_tol", 1e-8), n_alpha_bounds=kw.get("n_alpha_bounds", 10),
               snap_tol=kw.get("snap_tol", 0.0), clip=kw.get("clip", True))
    gpu = capi.Simplic(mesh, record_cut_faces=1, **okw)
    return gpu, O.Oracle(mesh, **okw)


def _assert_same_reconstruction(g, o):
    gc, gs = g.mixed()
    oc, os_ = o.mixed()
    np.testing.assert_array_equal(gc, oc)
    np.testing.assert_array_equal(gs, os_)
    for a, b, name in zip(g.interface(), o.interface(), "NDCS"):
        np.testing.assert_array_equal(a, b, err_msg=f"interface{name}")


@pytest.mark.parametrize("kind,n", [("hex", 8), ("jitter", 8), ("tet", 5), ("checker", 6)])
def test_face_flatness_bitexact(kind, n):
    m = _mesh(kind, n)
    g, o = _pair(m)
    np.testing.assert_array_equal(g.face_flatness(), o.face_flatness())


@pytest.mark.parametrize("kind,n", [("hex", 16), ("jitter", 12), ("tet", 8), ("refined", 12), ("checker", 10)])
def test_reconstruct_bitexact(kind, n):
    m = _mesh(kind, n)
    a = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    g, o = _pair(m)
    g.reconstruct(a)
    o.reconstruct(a)
    _assert_same_reconstruction(g, o)
    assert len(g.mixed()[0]) > 0


def _run(mesh, flow, alpha0, steps, dt, **kw):
    g, o = _pair(mesh, **kw)
    ag = alpha0.copy()
    ao = alpha0.copy()
    vol0 = float(np.sum(alpha0 * mesh.V))
    t = 0.0
    for s in range(steps):
        t += dt
        fl = flow.at(t, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        _assert_same_reconstruction(g, o)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        assert np.max(np.abs(ag - ao)) <= ALPHA_TOL, f"step {s}"
        np.testing.assert_array_equal(ag, ao, err_msg=f"alpha step {s}")
        np.testing.assert_array_equal(g.cut_faces(), o.cut_faces(), err_msg=f"cut faces step {s}")
        np.testing.assert_array_equal(g.alpha_phi(), o.alpha_phi(), err_msg=f"alphaPhi step {s}")
    drift = abs(float(np.sum(ag * mesh.V)) - vol0) / vol0
    return ag, drift, g


@pytest.mark.parametrize("kind,n,steps", [("hex", 24, 12), ("jitter", 14, 8), ("tet", 8, 8), ("refined", 16, 10),
                                          ("checker", 12, 10)])
def test_deformation_steps_bitexact(kind, n, steps):
    m = _mesh(kind, n)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    _, drift, g = _run(m, flow, a0, steps, dt, n_alpha_bounds=3, clip=False)
    assert drift <= 1e-12


def test_bounding_heavy_bitexact():
    """Many overshooting cells per pass: exercises the dependency-level
    schedule of the bounding kernel against the serial reference loop."""
    m = _mesh("hex", 40)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    g, o = _pair(m, n_alpha_bounds=10, clip=False)
    ag, ao = a0.copy(), a0.copy()
    t = 0.0
    bounded = 0
    for s in range(10):
        t += dt
        fl = flow.at(t, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        np.testing.assert_array_equal(ag, ao, err_msg=f"alpha step {s}")
        np.testing.assert_array_equal(g.alpha_phi(), o.alpha_phi(), err_msg=f"alphaPhi step {s}")
        bounded = max(bounded, g.stats()[2])
    assert bounded >= 20  # the schedule really ran with many cells


def test_translation_steps_bitexact():
    m = _mesh("hex", 20)
    a0 = H.sphere_alpha(m, (0.25, 0.25, 0.25), 0.15)
    flow = H.TranslationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    _run(m, flow, a0, 10, dt)


def test_clip_and_snap_bitexact():
    m = _mesh("hex", 16)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = 1.5 * H.cfl_delta_t(m, flow.phi0)  # overshoots trigger bounding
    _run(m, flow, a0, 6, dt, n_alpha_bounds=2, snap_tol=1e-6, clip=True)


def test_sources_bitexact():
    m = _mesh("hex", 12)
    a0 = H.sphere_alpha(m, (0.5, 0.5, 0.5), 0.2)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    rng = np.random.default_rng(3)
    Sp = -rng.uniform(0, 0.1, m.n_cells)
    Su = rng.uniform(0, 0.01, m.n_cells)
    g, o = _pair(m)
    fl = flow.at(dt, dt)
    g.reconstruct(a0)
    o.reconstruct(a0)
    ag = g.advect(a0, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, Sp=Sp, Su=Su)
    ao = o.advect(a0, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, Sp=Sp, Su=Su)
    np.testing.assert_array_equal(ag, ao)


def test_alpha_old_and_boundary_alpha():
    m = _mesh("hex", 12)
    a0 = H.sphere_alpha(m, (0.3, 0.5, 0.5), 0.25)
    flow = H.TranslationFlow(m, U=(1.0, 0.2, 0.1))
    dt = H.cfl_delta_t(m, flow.phi0)
    a_old = np.clip(a0 * 0.98, 0, 1)
    ab = np.zeros(m.n_boundary_faces)
    ab[::7] = 1.0
    g, o = _pair(m)
    fl = flow.at(dt, dt)
    g.reconstruct(a0)
    o.reconstruct(a0)
    ag = g.advect(a0, fl.phi, fl.U, dt, alpha_old=a_old, U_boundary=fl.U_boundary, alpha_boundary=ab)
    ao = o.advect(a0, fl.phi, fl.U, dt, alpha_old=a_old, U_boundary=fl.U_boundary, alpha_boundary=ab)
    np.testing.assert_array_equal(ag, ao)
    np.testing.assert_array_equal(g.alpha_phi(), o.alpha_phi())


def test_rho_phi():
    m = _mesh("hex", 10)
    a0 = H.sphere_alpha(m, (0.5, 0.5, 0.5), 0.3)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    g, _ = _pair(m)
    fl = flow.at(dt, dt)
    g.reconstruct(a0)
    g.advect(a0, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
    rp = g.rho_phi(1000.0, 1.0, fl.phi)
    np.testing.assert_array_equal(rp, (1000.0 - 1.0) * g.alpha_phi() + 1.0 * fl.phi)


def test_mesh_structure_found_at_create():
    """The update reads no face-slot records for the interior cells of a
    single-block lattice; the mixed forms solve box cells in closed form.
    Both are found at create and only when they hold for every cell."""
    hexm = mg.make_mesh("hex", 12)
    assert capi.Simplic(hexm).mesh_info() == (6, 12, 12, 12, 12 ** 3)
    jit = mg.make_mesh("jitter", 12)
    assert capi.Simplic(jit).mesh_info() == (6, 12, 12, 12, 0)
    tet = mg.make_mesh("tet", 6)
    assert capi.Simplic(tet).mesh_info() == (4, 0, 0, 0, 0)



@pytest.mark.parametrize("kind,n,steps", [("jitter", 12, 6), ("hex", 12, 4)])
def test_split_warped_face_bitexact(kind, n, steps):
    """splitWarpedFace true (cutCell.C:140-236): warped faces of the
    jittered mesh become triangle fans about their centres, whose centres
    join the vertex levels of the plane solve; on the flat hex mesh only the
    neighbour-side reversal of the faces changes the arithmetic."""
    m = _mesh(kind, n)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    okw = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=False)
    g = capi.Simplic(m, split_warped_face=1, record_cut_faces=1, **okw)
    o = O.Oracle(m, split_warped_face=True, **okw)
    ag, ao = a0.copy(), a0.copy()
    for s in range(steps):
        fl = flow.at((s + 1) * dt, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        _assert_same_reconstruction(g, o)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        np.testing.assert_array_equal(ag, ao, err_msg=f"alpha step {s}")


def test_pinned_velocity_is_read_in_place():
    """advect with U / U_boundary in pinned host memory (read in place by
    the interface kernels) equals the copied (pageable) path bit for bit."""
    torch = pytest.importorskip("torch")
    m = _mesh("hex", 20)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    fl = flow.at(dt, dt)
    tU = torch.empty((m.n_cells, 3), dtype=torch.float64, pin_memory=True)
    tUb = torch.empty((m.n_boundary_faces, 3), dtype=torch.float64, pin_memory=True)
    tU.numpy()[:] = fl.U
    tUb.numpy()[:] = fl.U_boundary
    outs = []
    for U, Ub in ((fl.U, fl.U_boundary), (tU.numpy(), tUb.numpy())):
        g = capi.Simplic(m, n_alpha_bounds=3, clip=0)
        g.reconstruct(a0)
        outs.append((g.advect(a0, fl.phi, U, dt, U_boundary=Ub, unchanged=True), g.alpha_phi()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("case", ["empty", "full", "one-cell", "slab"])
def test_degenerate_fields_bitexact(case):
    """Fields without an interface or with a minimal one, on a 32^3 lattice
    (the update's lattice path) in the deformation field: every cell empty,
    every cell full, one cell at alpha 0.3 in an empty domain, and a flat
    slab alpha = 1 for z < 0.5 (an interface of planar cells only, no
    Simpson flux across a cell with a tilted plane).  Plain form bit for
    bit with the oracle over 4 steps; the learned form runs the same steps
    (a network stage with zero or few rows) and keeps the volume."""
    from geometricvofext_gb300 import mlp

    mesh = _mesh("hex", 32)
    if case == "empty":
        a0 = np.zeros(mesh.n_cells)
    elif case == "full":
        a0 = np.ones(mesh.n_cells)
    elif case == "one-cell":
        a0 = np.zeros(mesh.n_cells)
        a0[16 + 32 * (16 + 32 * 16)] = 0.3
    else:
        a0 = (mesh.C[:, 2] < 0.5).astype(np.float64)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    g, o = _pair(mesh, n_alpha_bounds=3, clip=False)
    gl = capi.Simplic(mesh, precision=capi.PRECISION_LEARNED, n_alpha_bounds=3, clip=0)
    gl.set_network(*mlp.load_weights())
    ag, ao, al = a0.copy(), a0.copy(), a0.copy()
    for s in range(4):
        fl = flow.at((s + 1) * dt, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        _assert_same_reconstruction(g, o)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        np.testing.assert_array_equal(ag, ao)
        np.testing.assert_array_equal(g.alpha_phi(), o.alpha_phi())
        gl.reconstruct(al)
        al = gl.advect(al, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
    if case == "empty":
        assert not ag.any() and not al.any()
    v0 = float(np.sum(a0 * mesh.V))
    if v0 > 0:
        assert abs(float(np.sum(al * mesh.V)) - v0) <= 1e-12 * v0
