"""isoRDF orientation (reconstruction.C:193-405) on the GPU against the CPU
oracle, through the C ABI.

The plain form's isoRDF loop reproduces the oracle's: normals, plane
constants, interface centres and areas, cell statuses and, over advection
steps, alpha -- bit for bit.  The iteration count depends on residual sums
that include acos() of the angles between neighbouring normals (CUDA's and
the C library's acos may differ in the last bit); the sums only meet
thresholds, so the counts agree except at an exact tie, which these cases
do not hit.  The reconstructed distance function is restated from the
published method (OpenFOAM's own is absent), identically on both sides.
"""

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CTRL = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=0)


def _pair(mesh, **kw):
    g = capi.Simplic(mesh, orientation_method=capi.ORIENTATION_ISO_RDF, record_cut_faces=1, **CTRL, **kw)
    o = O.Oracle(mesh, orientation="isoRDF", n_threads=8, **dict(CTRL, clip=False))
    return g, o


@pytest.mark.parametrize("kind,n", [("hex", 20), ("jitter", 14), ("tet", 8), ("checker", 10)])
def test_rdf_reconstruct_bitexact(kind, n):
    m = mg.make_mesh(kind, n)
    a = H.sphere_alpha(m, (0.45, 0.5, 0.55), 0.27)
    g, o = _pair(m)
    g.reconstruct(a)
    o.reconstruct(a)
    gc, gs = g.mixed()
    oc, os_ = o.mixed()
    np.testing.assert_array_equal(gc, oc)
    np.testing.assert_array_equal(gs, os_)
    for x, y, name in zip(g.interface(), o.interface(), "NDCS"):
        np.testing.assert_array_equal(x, y, err_msg=f"interface{name}")
    assert g.rdf_iterations() == o.rdf_iterations() >= 2


@pytest.mark.parametrize("kind,n,steps", [("hex", 24, 10), ("tet", 8, 6)])
def test_rdf_deformation_steps_bitexact(kind, n, steps):
    m = mg.make_mesh(kind, n)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    g, o = _pair(m)
    ag, ao = a0.copy(), a0.copy()
    for k in range(steps):
        fl = flow.at((k + 1) * dt, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        np.testing.assert_array_equal(ag, ao, err_msg=f"step {k}")
        np.testing.assert_array_equal(g.alpha_phi(), o.alpha_phi(), err_msg=f"alphaPhi step {k}")
    v0 = float(np.sum(a0 * m.V))
    assert abs(float(np.sum(ag * m.V)) - v0) / v0 <= 1e-12


def test_rdf_normals_beat_least_squares_and_compare_with_the_network():
    """On a sphere (R = 0.27 on 32^3 hexes) the isoRDF normals are closer to
    the exact sphere normals than the least-squares ones; the learned
    form's normals are reported beside them (the network is the other way
    to better normals)."""
    from geometricvofext_gb300 import mlp

    m = mg.make_mesh("hex", 32)
    c0 = np.array((0.45, 0.5, 0.55))
    a = H.sphere_alpha(m, c0, 0.27)
    err = {}
    for name, kw in (("ls", {}), ("rdf", {"orientation_method": capi.ORIENTATION_ISO_RDF}),
                     ("learned", {"precision": capi.PRECISION_LEARNED})):
        g = capi.Simplic(m, **CTRL, **kw)
        if name == "learned":
            g.set_network(*mlp.load_weights())
        g.reconstruct(a)
        cells, st = g.mixed()
        N, _, Cc, _ = g.interface()
        sel = cells[st == 0]
        ex = Cc[sel] - c0
        ex /= np.linalg.norm(ex, axis=1)[:, None]
        err[name] = float(np.degrees(np.arccos(np.clip(np.sum(N[sel] * ex, axis=1), -1, 1))).mean())
    assert err["rdf"] < 0.5 * err["ls"], err
    assert err["learned"] < err["ls"], err
    print("mean normal error (deg):", err)
