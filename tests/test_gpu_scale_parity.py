"""Bit-exact parity of the plain FP64 form with the CPU oracle at the sizes the
benchmark and the unstructured-mesh configurations use (host-buffer C ABI,
the drop-in path).

* the benchmark workload itself: 256^3 hex (16.8 M cells), deformation field
  T = 6, sphere R = 0.15 at (0.35, 0.35, 0.35), Courant 0.5, the reference
  test's controls (nAlphaBounds 3, clip off), first 10 steps;
* the unstructured meshes: 96^3 hex with interior points jittered by
  +-0.2 h (seed 12345, non-planar faces) and 64^3 hexes split into 6 tets
  (1,572,864 cells), 20 steps each of the same deformation case;
* the 128^3 deformation case over its whole period t = 0 .. 3 (1904 steps),
  where the shape returns.

Every step compares alpha, alphaPhi, the ascending mixed-cell list with the
cell statuses and the mask of Simpson-integrated faces by exact equality
(the plain form reproduces the oracle's doubles bit for bit); the interface
planes (interfaceN/D/C/S) are compared on the steps listed per case.  The
oracle is the restatement of the reference's CPU algorithm; OpenFOAM's own
pieces on the path (cell-point interpolation, least-squares gradient,
stencil order) are restated identically on both sides and are not pinned to
OpenFOAM itself.
"""

import math
import os

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CTRL = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=False)
THREADS = os.cpu_count() or 1


def _compare_step(g, o, k, interface=False):
    gc, gs = g.mixed()
    oc, os_ = o.mixed()
    np.testing.assert_array_equal(gc, oc, err_msg=f"mixed cells, step {k}")
    np.testing.assert_array_equal(gs, os_, err_msg=f"cell status, step {k}")
    if interface:
        for a, b, name in zip(g.interface(), o.interface(), "NDCS"):
            np.testing.assert_array_equal(a, b, err_msg=f"interface{name}, step {k}")


def _lockstep(mesh, flow, alpha0, dt, steps, interface_steps=(), check_every=1):
    """Both solvers from the same field; returns the final alphas."""
    g = capi.Simplic(mesh, record_cut_faces=1, **CTRL)
    o = O.Oracle(mesh, n_threads=THREADS, **CTRL)
    ag, ao = alpha0.copy(), alpha0.copy()
    for k in range(steps):
        fl = flow.at((k + 1) * dt, dt)
        g.reconstruct(ag)
        o.reconstruct(ao)
        full = (k % check_every == 0) or k == steps - 1
        if full or k in interface_steps:
            _compare_step(g, o, k, interface=k in interface_steps)
        ag = g.advect(ag, fl.phi, fl.U, dt, U_boundary=fl.U_boundary, unchanged=True)
        ao = o.advect(ao, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        np.testing.assert_array_equal(ag, ao, err_msg=f"alpha, step {k}")
        if full:
            np.testing.assert_array_equal(g.alpha_phi(), o.alpha_phi(), err_msg=f"alphaPhi, step {k}")
            np.testing.assert_array_equal(g.cut_faces(), o.cut_faces(), err_msg=f"cut faces, step {k}")
    return ag, ao, g


def _deformation_case(mesh):
    alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    return alpha0, flow, dt


def test_benchmark_workload_256_first_10_steps_bitexact():
    mesh = mg.hex_mesh(256)
    alpha0, flow, dt = _deformation_case(mesh)
    ag, _, g = _lockstep(mesh, flow, alpha0, dt, 10, interface_steps=(9,))
    vol0 = float(np.sum(alpha0 * mesh.V))
    assert abs(float(np.sum(ag * mesh.V)) - vol0) / vol0 <= 1e-12
    assert g.stats()[0] > 20000  # the interface of the benchmark step


@pytest.mark.parametrize("kind,n", [("jitter", 96), ("tet", 64)])
def test_unstructured_meshes_20_steps_bitexact(kind, n):
    mesh = mg.make_mesh(kind, n, seed=12345)
    if kind == "tet":
        assert mesh.n_cells == 1572864
    alpha0, flow, dt = _deformation_case(mesh)
    ag, _, g = _lockstep(mesh, flow, alpha0, dt, 20, interface_steps=(0, 19))
    vol0 = float(np.sum(alpha0 * mesh.V))
    assert abs(float(np.sum(ag * mesh.V)) - vol0) / vol0 <= 1e-12
    assert g.stats()[0] > 1000


def test_deformation_128_full_period_bitexact():
    """All 1904 steps of the 128^3 case: alpha compared at every step, the
    classification, alphaPhi and cut faces every 50 steps and at the end."""
    mesh = mg.hex_mesh(128)
    alpha0, flow, dt = _deformation_case(mesh)
    steps = int(math.ceil(3.0 / dt - 1e-9))
    dt = 3.0 / steps
    ag, _, _ = _lockstep(mesh, flow, alpha0, dt, steps, interface_steps=(steps // 2,), check_every=50)
    vol0 = float(np.sum(alpha0 * mesh.V))
    e = H.errors(ag, alpha0, mesh.V, vol0)
    assert abs(e.volume_error) <= 1e-12
    assert e.shape_error < 0.15  # the shape is back (0.104 at 128^3 with LS normals)
