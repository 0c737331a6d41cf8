"""Known-answer tests of the CPU oracle (restatement of the reference's
cutFace / cutCell / reconstruction / advection) -- no GPU needed."""

import itertools

import numpy as np
import pytest

from geometricvofext_gb300 import harness as H, meshgen as mg
from oracle import oracle as O


def cube_fraction_below(n, c):
    """Volume of {x in [0,1]^3 : n.x <= c} (inclusion-exclusion over the
    cube vertices; all n_i must be nonzero)."""
    n = np.asarray(n, float)
    flip = n < 0
    c = c - np.sum(n[flip])
    m = np.abs(n)
    tot = 0.0
    for v in itertools.product((0, 1), repeat=3):
        s = c - float(np.dot(m, v))
        if s > 0:
            tot += (-1) ** sum(v) * s ** 3
    return tot / (6.0 * m[0] * m[1] * m[2])


@pytest.fixture(scope="module")
def cube():
    m = mg.hex_mesh(1)
    return m, O.Oracle(m)


def test_cube_cut_vof_matches_analytic(cube):
    m, o = cube
    rng = np.random.default_rng(7)
    for _ in range(200):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        if np.min(np.abs(n)) < 1e-3:
            continue
        lo, hi = min(0.0, n.sum()) + min(n.min(), 0), max(n[n > 0].sum(), 0)
        c = rng.uniform(np.sum(np.minimum(n, 0)), np.sum(np.maximum(n, 0)))
        st, vof, ic, isv = o.calc_sub_cell(0, n, -c)  # submerged: x.n + d < 0 -> n.x < c
        exp = cube_fraction_below(n, c)
        assert abs(vof - exp) < 1e-13, (n, c, vof, exp)
        if 1e-9 < exp < 1 - 1e-9:
            assert st == 0
            # interface area vector is parallel to the normal
            assert abs(abs(np.dot(isv, n)) - np.linalg.norm(isv)) < 1e-12


def test_axis_aligned_cut(cube):
    m, o = cube
    for z in (0.1, 0.5, 0.93):
        st, vof, ic, isv = o.calc_sub_cell(0, np.array([0.0, 0.0, 1.0]), -z)
        assert st == 0 and abs(vof - z) < 1e-15
        np.testing.assert_allclose(ic, [0.5, 0.5, z], atol=1e-15)
        np.testing.assert_allclose(isv, [0, 0, 1.0], atol=1e-15)


@pytest.mark.parametrize("kind,n,tol", [("hex", 3, 1e-12), ("tet", 2, 1e-12), ("jitter", 3, 2e-3)])
def test_find_signed_distance_inverts_vof(kind, n, tol):
    """Exact (to round-off) on planar-faced cells, where the submerged volume
    is a cubic in d between vertex levels; on warped faces the reference's
    cubic fit is only approximate (cutCell.C:743-789)."""
    m = mg.make_mesh(kind, n)
    o = O.Oracle(m)
    rng = np.random.default_rng(11)
    for cell in range(0, m.n_cells, max(1, m.n_cells // 9)):
        for _ in range(6):
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            a = rng.uniform(0.01, 0.99)
            st, d, c, s = o.find_signed_distance(cell, a, nrm)
            st2, vof, _, _ = o.calc_sub_cell(cell, nrm, d)
            assert st == 0 and st2 == 0
            assert abs(vof - a) < tol, (kind, cell, a, vof)


def test_zero_normal_status(cube):
    m, o = cube
    assert o.find_signed_distance(0, 0.3, np.zeros(3))[0] == 1
    assert o.find_signed_distance(0, 0.7, np.zeros(3))[0] == -1


def test_calc_sub_face_square():
    sq = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], float)
    st, c, a = O.calc_sub_face(sq, np.array([1.0, 0, 0]), -0.25)
    assert st == 0
    np.testing.assert_allclose(a, [0, 0, 0.25], atol=1e-15)
    np.testing.assert_allclose(c, [0.125, 0.5, 0], atol=1e-15)
    assert O.calc_sub_face(sq, np.array([1.0, 0, 0]), -2.0)[0] == -1
    assert O.calc_sub_face(sq, np.array([1.0, 0, 0]), 2.0)[0] == 1
    # diagonal cut: triangle of area 1/2 * 0.5^2
    n = np.array([1.0, 1.0, 0]) / np.sqrt(2)
    st, c, a = O.calc_sub_face(sq, n, -0.5 / np.sqrt(2))
    assert abs(np.linalg.norm(a) - 0.125) < 1e-15


def test_time_integrated_face_flux_limits():
    m = mg.hex_mesh(2)
    o = O.Oracle(m)
    f = 0  # +x face at x = 0.5 of cell 0
    np.testing.assert_allclose(m.Sf[f], [0.25, 0, 0])
    magSf = m.magSf[f]
    n = np.array([1.0, 0, 0])
    phi, dt = 0.3, 0.1
    # stationary interface at x = 0.3: face empty -> 0 ; at x = 0.7: full
    assert o.time_integrated_face_flux(f, n, -0.3, 0.0, dt, phi, magSf) == 0.0
    assert abs(o.time_integrated_face_flux(f, n, -0.7, 0.0, dt, phi, magSf) - phi * dt) < 1e-16
    # interface normal to x, moving +x at speed 1, starting at x = 0.45:
    # reaches the face at tau = 0.05, then the face is full for the rest
    v = o.time_integrated_face_flux(f, n, -0.45, 1.0, dt, phi, magSf)
    assert abs(v - phi * 0.05) < 1e-14
    # tiny flux -> zero
    assert o.time_integrated_face_flux(f, n, -0.45, 1.0, dt, 1e-15, magSf) == 0.0
    # oblique plane sweeping a face: Simpson on a quadratic area is exact
    n2 = np.array([1.0, 1.0, 0.0]) / np.sqrt(2)
    Un0 = 0.4
    v = o.time_integrated_face_flux(f, n2, -0.5 / np.sqrt(2) * 1.6, Un0, dt, phi, magSf)
    ts = np.linspace(0, dt, 20001)
    areas = []
    for t in ts:
        dd = -0.5 / np.sqrt(2) * 1.6 - t * Un0
        # face x=0.5, y,z in [0,0.5]: submerged where (0.5 + y)/sqrt2 + dd < 0
        ylim = np.clip(-dd * np.sqrt(2) - 0.5, 0, 0.5)
        areas.append(ylim * 0.5)
    ref = phi / magSf * np.trapezoid(areas, ts)
    assert abs(v - ref) < 1e-9


def test_interpolate_uniform_U():
    m = mg.make_mesh("jitter", 4)
    o = O.Oracle(m)
    U = np.tile([0.3, -0.2, 0.7], (m.n_cells, 1))
    Ub = np.tile([0.3, -0.2, 0.7], (m.n_boundary_faces, 1))
    rng = np.random.default_rng(1)
    for c in range(0, m.n_cells, 5):
        x = m.C[c] + rng.uniform(-0.2, 0.2, 3) * m.h
        np.testing.assert_allclose(o.interpolate_U(c, x, U, Ub), [0.3, -0.2, 0.7], atol=1e-14)


def test_ls_normal_of_planar_interface():
    m = mg.hex_mesh(12)
    o = O.Oracle(m)
    nrm = np.array([0.4, 0.5, 0.7])
    nrm /= np.linalg.norm(nrm)
    c0 = float(nrm @ [0.5, 0.5, 0.5])
    # exact cut-cell fractions of the half-space n.x < c0
    a = np.array([o.calc_sub_cell(c, nrm, -c0)[1] for c in range(m.n_cells)])
    o.reconstruct(a)
    cells, st = o.mixed()
    n, d, cc, s = o.interface()
    interior = [c for c in cells if np.all(np.abs(m.C[c] - 0.5) < 0.3)]
    assert len(interior) > 10
    # the LS normal points from liquid to gas: +nrm
    cosang = n[interior] @ nrm
    assert np.min(cosang) > 0.995


def _steps(mesh, a0, flow, dt, steps, **kw):
    o = O.Oracle(mesh, **kw)
    a = a0.copy()
    t = 0.0
    for _ in range(steps):
        t += dt
        fl = flow.at(t, dt)
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
    return a


def test_conservation_and_boundedness():
    m = mg.hex_mesh(16)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    a = _steps(m, a0, flow, dt, 15, n_alpha_bounds=3, clip=False)
    v0, v1 = np.sum(a0 * m.V), np.sum(a * m.V)
    assert abs(v1 - v0) / v0 <= 1e-12
    assert a.min() > -1e-6 and a.max() < 1 + 1e-6


def test_serial_equals_openmp():
    m = mg.hex_mesh(14)
    a0 = H.sphere_alpha(m, (0.4, 0.45, 0.5), 0.2)
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    a1 = _steps(m, a0, flow, dt, 6, n_threads=1)
    a4 = _steps(m, a0, flow, dt, 6, n_threads=4)
    np.testing.assert_array_equal(a1, a4)


def test_translation_moves_the_sphere():
    m = mg.hex_mesh(24)
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    flow = H.TranslationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    steps = 12
    a = _steps(m, a0, flow, dt, steps)
    cen0 = (a0 * m.V) @ m.C / np.sum(a0 * m.V)
    cen1 = (a * m.V) @ m.C / np.sum(a * m.V)
    np.testing.assert_allclose(cen1 - cen0, 0.5 * steps * dt * np.ones(3), atol=0.05 * m.h)


def test_spheres_and_slab_case():
    """The scale case's initial field (a seeded union of spheres plus the slab
    z < 0.2, here on 48^3 with radii of a few cells): its volume is the
    spheres' plus the slab's, and the oracle advects it conservatively and
    boundedly in the deformation field."""
    m = mg.hex_mesh(48)
    a0 = H.spheres_and_slab_alpha(m, n_spheres=12, rmin=0.05, rmax=0.08)
    assert a0.min() >= 0.0 and a0.max() <= 1.0
    vol = float(np.sum(a0 * m.V))
    # the slab is exact; each sphere's fraction comes from the cell-box overlap
    assert 0.2 < vol < 0.2 + 12 * 4.0 / 3.0 * np.pi * 0.08 ** 3 + 1e-9
    n_mixed = int(np.count_nonzero((a0 > 1e-8) & (a0 < 1 - 1e-8)))
    assert n_mixed > 48 * 48  # the slab's layer plus the spheres' shells
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    a = _steps(m, a0, flow, dt, 4, n_alpha_bounds=3, clip=False)
    assert abs(np.sum(a * m.V) - vol) / vol <= 1e-12
    # three bounding passes without clipping leave overshoots of order 1e-6
    # (the reference case reports min alpha and 1 - max alpha as metrics)
    assert a.min() > -1e-4 and a.max() < 1 + 1e-4


@pytest.mark.parametrize("kind,n", [("refined", 12), ("checker", 10)])
def test_refined_meshes_and_the_oracle_on_them(kind, n):
    """The 2:1-refined meshes (a refined box; every other cell of a box
    refined): closed cells, the unit volume, and cells as large as the
    static caps allow -- transition cells with up to 24 faces and 26 points,
    faces with up to 8 points (hanging nodes).  The oracle advances a
    sphere on them with the volume kept to round-off."""
    m = mg.make_mesh(kind, n)
    offs, _ = m.cell_faces()
    nfc = np.diff(offs)
    S = np.zeros((m.n_cells, 3))
    np.add.at(S, m.owner, m.Sf)
    np.add.at(S, m.neighbour, -m.Sf[:m.n_internal_faces])
    assert np.abs(S).max() < 1e-15 and abs(m.V.sum() - 1.0) < 1e-14
    if kind == "checker":
        assert nfc.max() == 24 and np.diff(m.face_offsets).max() == 8
        assert set(np.unique(nfc)) >= {6, 9, 15, 18, 21, 24}
    else:
        assert set(np.unique(nfc)) == {6, 9}
    a0 = H.sphere_alpha(m, (0.45, 0.5, 0.55), 0.27)
    assert abs(float(np.sum(a0 * m.V)) - 4.0 / 3.0 * np.pi * 0.27 ** 3) < 1e-9
    flow = H.DeformationFlow(m)
    dt = H.cfl_delta_t(m, flow.phi0)
    o = O.Oracle(m, n_alpha_bounds=3, clip=False)
    a = a0.copy()
    for k in range(6):
        fl = flow.at((k + 1) * dt, dt)
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
    v0 = float(np.sum(a0 * m.V))
    assert abs(float(np.sum(a * m.V)) - v0) / v0 < 1e-13
    assert a.min() > -1e-9 and a.max() < 1 + 1e-9
