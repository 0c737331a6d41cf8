"""PLIC surface extraction (reconstruction::interface, reconstruction.C:787-835;
cutCell::interfacePoints, cutCell.C:545-608).

CPU: the oracle's polygons are closed planar fans of the cell's interface
plane whose area equals the interface area of the plane solve, and the VTP
writer round-trips them.  GPU: the CUDA polygons equal the oracle's (points
bit for bit, same order, same cells) on hexahedra, jittered hexahedra,
tetrahedra and 2:1-refined cells, and with the isoRDF orientation.
"""

import os

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg, plic_surface as PS
from oracle import oracle as O


def _polygon_area(P):
    c = P.mean(axis=0)
    return 0.5 * np.sum(np.cross(P - c, np.roll(P, -1, axis=0) - c), axis=0)


@pytest.mark.parametrize("kind,n", [("hex", 16), ("tet", 7)])
def test_oracle_polygons_lie_in_the_planes(kind, n):
    m = mg.make_mesh(kind, n)
    a = H.sphere_alpha(m, (0.5, 0.5, 0.5), 0.3)
    o = O.Oracle(m)
    o.reconstruct(a)
    off, pts, cells = o.interface_polygons()
    N, D, Cc, S = o.interface()
    _, st = o.mixed()
    assert cells.size == int(np.sum(st == 0)) and np.all(np.diff(cells) > 0)
    for k, c in enumerate(cells):
        P = pts[off[k]:off[k + 1]]
        assert P.shape[0] >= 3
        assert np.max(np.abs(P @ N[c] + D[c])) < 1e-12
        A = _polygon_area(P)
        # the ordered polygon's area is the interface area of the cut
        assert np.linalg.norm(A - S[c] * np.sign(A @ S[c])) < 1e-9 * max(1.0, np.linalg.norm(S[c])) + 1e-14


def test_vtp_round_trip(tmp_path):
    m = mg.make_mesh("hex", 10)
    a = H.sphere_alpha(m, (0.5, 0.5, 0.5), 0.3)
    o = O.Oracle(m)
    o.reconstruct(a)
    off, pts, cells = o.interface_polygons()
    path = os.path.join(tmp_path, "plic.vtp")
    PS.write_vtp(path, off, pts, cells, {"alpha.water": a, "U": m.C})
    off2, pts2, data = PS.read_vtp(path)
    np.testing.assert_array_equal(off2, off)
    np.testing.assert_array_equal(pts2, pts)
    np.testing.assert_array_equal(data["cellIds"], cells)
    np.testing.assert_array_equal(data["alpha.water"], a[cells])
    np.testing.assert_array_equal(data["U"], m.C[cells])


@pytest.mark.gpu
@pytest.mark.parametrize("kind,n,orient", [("hex", 16, "isoAlphaGrad"), ("jitter", 12, "isoAlphaGrad"),
                                           ("tet", 7, "isoAlphaGrad"), ("checker", 10, "isoAlphaGrad"),
                                           ("hex", 16, "isoRDF")])
def test_gpu_polygons_equal_the_oracle(kind, n, orient):
    m = mg.make_mesh(kind, n)
    a = H.sphere_alpha(m, (0.45, 0.5, 0.55), 0.27)
    om = capi.ORIENTATION_ISO_RDF if orient == "isoRDF" else capi.ORIENTATION_ISO_ALPHA_GRAD
    g = capi.Simplic(m, orientation_method=om)
    o = O.Oracle(m, orientation=orient)
    g.reconstruct(a)
    o.reconstruct(a)
    for x, y in zip(g.interface_polygons(), o.interface_polygons()):
        np.testing.assert_array_equal(x, y)
    # a second request returns the cached surface
    off, pts, cells = g.interface_polygons()
    assert cells.size > 0 and off[-1] == pts.shape[0]
