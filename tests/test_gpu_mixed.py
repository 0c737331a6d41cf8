"""Mixed-precision form against the FP64 oracle.

The mixed form computes interface normals and the Simpson face clipping in
FP32 and the plane constant in FP64 (the closed-form cuboid inverse on box
cells, the reference's bracket and cubic elsewhere).  It is not bit-exact by
design; what it must keep:

* the mixed-cell classification (the same FP64 scan);
* the cell volume: the oracle's own cutCell::calcSubCell on the mixed form's
  plane gives back alpha within 1e-11, or as closely as the plain form's
  plane does (the reference's cubic is exact only where the cut volume is a
  cubic in the plane constant: cells with planar faces);
* normals within 1e-4 rad of the FP64 least-squares normals;
* mass conservation to 1e-12 relative and boundedness like the plain form;
* the L1 shape error of a deformation run within a few percent of the plain
  form's.
"""

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CTRL = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=False)


def _pair(mesh):
    gm = capi.Simplic(mesh, precision=capi.PRECISION_MIXED, **CTRL)
    gp = capi.Simplic(mesh, precision=capi.PRECISION_PLAIN_FP64, **CTRL)
    return gm, gp


@pytest.mark.parametrize("kind,n", [("hex", 16), ("jitter", 12), ("tet", 8)])
def test_mixed_plane_matches_cell_volume(kind, n):
    mesh = mg.make_mesh(kind, n)
    a = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    gm, gp = _pair(mesh)
    gm.reconstruct(a)
    gp.reconstruct(a)
    cm, sm = gm.mixed()
    cp, sp = gp.mixed()
    np.testing.assert_array_equal(cm, cp)
    nm, dm, icm, ism = gm.interface()
    npl, dpl, _, _ = gp.interface()
    o = O.Oracle(mesh, **CTRL)
    worst = worst_c = worst_s = worst_plain = 0.0
    h = np.cbrt(mesh.V.mean())
    for c in cm:
        st, vof, ic, isv = o.calc_sub_cell(c, nm[c], dm[c])
        worst = max(worst, abs(vof - a[c]))
        worst_c = max(worst_c, np.abs(np.asarray(ic) - icm[c]).max() / h)
        worst_s = max(worst_s, np.abs(np.asarray(isv) - ism[c]).max() / h**2)
        worst_plain = max(worst_plain, abs(o.calc_sub_cell(c, npl[c], dpl[c])[1] - a[c]))
    assert worst <= max(1e-11, 2.0 * worst_plain), (worst, worst_plain)
    # interface centre (FP32 clipping on box cells) and area vector at that plane
    assert worst_c <= 1e-5, worst_c
    assert worst_s <= 1e-9, worst_s
    # FP32 normals: direction within 1e-4 rad of the FP64 least-squares normal
    dots = np.einsum("ij,ij->i", nm[cm], npl[cm])
    ang = np.arccos(np.clip(dots / (np.linalg.norm(nm[cm], axis=1) * np.linalg.norm(npl[cm], axis=1)), -1, 1))
    assert ang.max() < 1e-4, ang.max()


def _run(g, mesh, flow, alpha0, steps, dt):
    a = alpha0.copy()
    t = 0.0
    for _ in range(steps):
        t += dt
        fl = flow.at(t, dt)
        g.reconstruct(a)
        a = g.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
    return a


@pytest.mark.parametrize("kind,n", [("hex", 24), ("tet", 10)])
def test_mixed_deformation_conserves_and_tracks_plain(kind, n):
    mesh = mg.make_mesh(kind, n)
    alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    gm, gp = _pair(mesh)
    steps = 40
    am = _run(gm, mesh, flow, alpha0, steps, dt)
    ap = _run(gp, mesh, flow, alpha0, steps, dt)
    vol0 = float(np.sum(alpha0 * mesh.V))
    em = H.errors(am, ap, mesh.V, vol0)
    drift = abs(float(np.sum(am * mesh.V)) - vol0) / vol0
    assert drift <= 1e-12, drift
    ep = H.errors(ap, ap, mesh.V, vol0)
    # boundedness like the plain form (bounding is the same FP64 kernel)
    assert em.boundedness <= max(ep.boundedness, 1e-12) + 1e-9, (em.boundedness, ep.boundedness)
    # the two forms stay close (L1 difference relative to the volume)
    assert em.shape_error < 2e-3, em.shape_error


def test_mixed_shape_error_full_period():
    """Deformation over t in [0, 3] (the field reverses at t = 1.5, the shape
    returns at t = 3): shape error of the mixed form within 5% of the plain
    form's, volume conserved to 1e-12."""
    mesh = mg.make_mesh("hex", 32)
    alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    steps = int(round(3.0 / dt))
    dt = 3.0 / steps
    gm, gp = _pair(mesh)
    am = _run(gm, mesh, flow, alpha0, steps, dt)
    ap = _run(gp, mesh, flow, alpha0, steps, dt)
    vol0 = float(np.sum(alpha0 * mesh.V))
    em = H.errors(am, alpha0, mesh.V, vol0)
    ep = H.errors(ap, alpha0, mesh.V, vol0)
    assert abs(em.volume_error) <= 1e-12
    assert em.shape_error <= 1.05 * ep.shape_error, (em.shape_error, ep.shape_error)


@pytest.mark.parametrize("kind,n", [("hex", 20), ("jitter", 12), ("tet", 8)])
def test_mixed_simpson_face_fluxes_match_fp64(kind, n):
    """The mixed form's Simpson fluxes face by face: for every downwind face
    of a cut cell, its dVf (alphaPhi * dt, no bounding) against the oracle's
    FP64 cutFace::timeIntegratedFaceFlux with the mixed form's own plane
    (normal, constant) and the FP64 interface speed U(interface centre) . n.
    The mixed form clips in FP32 on face-local coordinates and takes the
    interface speed and the vertex arrival times in FP32; the difference is
    bounded relative to the face's whole flux |phi| dt."""
    mesh = mg.make_mesh(kind, n)
    a = H.sphere_alpha(mesh, (0.45, 0.5, 0.55), 0.27)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    fl = flow.at(0.4, dt)
    ctrl = dict(CTRL, n_alpha_bounds=0)
    g = capi.Simplic(mesh, precision=capi.PRECISION_MIXED, **ctrl)
    g.reconstruct(a)
    g.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
    cells, st = g.mixed()
    nrm, dd, ic, _ = g.interface()
    aphi = g.alpha_phi()
    o = O.Oracle(mesh, **ctrl)
    own, nei, nfi = mesh.owner, mesh.neighbour, mesh.n_internal_faces
    faces_of = [[] for _ in range(mesh.n_cells)]
    for f in range(mesh.n_faces):
        faces_of[own[f]].append(f)
        if f < nfi:
            faces_of[nei[f]].append(f)
    worst, count = 0.0, 0
    for c, s in zip(cells, st):
        if s != 0:
            continue
        un0 = float(np.dot(o.interpolate_U(c, ic[c], fl.U, fl.U_boundary), nrm[c]))
        for f in faces_of[c]:
            ph = fl.phi[f]
            down = (ph >= 0.0) if own[f] == c else (ph < 0.0)
            if not down or abs(ph) <= 1e-14:
                continue
            ref = o.time_integrated_face_flux(f, nrm[c], dd[c], un0, dt, ph, mesh.magSf[f])
            worst = max(worst, abs(aphi[f] * dt - ref) / (abs(ph) * dt))
            count += 1
    assert count > 100
    assert worst <= 2e-5, worst
