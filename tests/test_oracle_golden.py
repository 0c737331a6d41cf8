"""The oracle and the workload generators pinned against the reference's own
data: the golden 64^3 "exact" fields of tutorials/test/exactSolutions (via
the permutation-invariant fixture tests/golden/exact64.npz, made by
tests/golden/make_golden.py) and exactInitialVol of
applications/test/calcVofAdvectionErrors/calcVofAdvectionErrors.C:64.

The golden fields are in the reference case's renumberMesh cell order, which
this project does not reproduce, so every comparison is permutation
invariant: volumes, mixed/full cell counts and sorted value distributions.
"""

import os

import numpy as np
import pytest

from geometricvofext_gb300 import harness as H, meshgen as mg
from oracle import oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "exact64.npz"))


def test_exact_initial_volume_constant():
    # sum(alpha) h^3 of the t=0 golden field is the constant the metric tool uses
    assert abs(GOLD["volume"][0] - H.EXACT_INITIAL_VOL_64) / H.EXACT_INITIAL_VOL_64 < 1e-10


def test_golden_fixture_shape_returns_at_t3():
    # the deformation field reverses: the t=3 field equals the t=0 field
    np.testing.assert_array_equal(GOLD["n_mixed"][0], GOLD["n_mixed"][-1])
    np.testing.assert_allclose(GOLD["sorted_t3"], GOLD["sorted_t0"], atol=1e-12)


@pytest.fixture(scope="module")
def mesh64():
    return mg.hex_mesh(64)


def test_sphere_init_matches_golden_t0(mesh64):
    """Our exact sphere overlap reproduces the reference's initial field up
    to the icosphere-vs-sphere difference: same interface/full cell counts,
    sorted fractions within 2e-4, volume within 5e-5 relative."""
    a = H.sphere_alpha(mesh64, (0.35, 0.35, 0.35), 0.15)
    tol = 1e-8
    assert int(np.count_nonzero((a > tol) & (a < 1 - tol))) == int(GOLD["n_mixed"][0])
    assert int(np.count_nonzero(a >= 1 - tol)) == int(GOLD["n_full"][0])
    nz = np.sort(a[a > 0])
    g = GOLD["sorted_t0"]
    assert nz.size == g.size
    assert np.max(np.abs(nz - g)) < 2e-4
    vol = float(np.sum(a * mesh64.V))
    assert abs(vol - GOLD["volume"][0]) / GOLD["volume"][0] < 5e-5
    # the analytic sphere volume
    assert abs(vol - 4.0 / 3.0 * np.pi * 0.15 ** 3) / vol < 1e-7


def test_golden_all_time_levels(mesh64):
    """The oracle run the way the reference test case runs (64^3, T = 6,
    adaptive step at Courant 0.5 landing on every 0.25 write time,
    nAlphaBounds 3, clip off), compared with the golden field at all 13
    write times t = 0, 0.25, ..., 3 with the error measures of
    applications/test/calcVofAdvectionErrors/updateErrors.H:9-31:

    * E_v(t) = (sum alpha V - exactInitialVol) / exactInitialVol
      (updateErrors.H:12): the sphere-vs-icosphere offset of the initial
      field (|E_v(0)| < 5e-5) and constant to 1e-12 relative afterwards;
    * minAlpha and 1 - maxAlpha (updateErrors.H:15-16) above -1e-6;
    * E_s (updateErrors.H:31) against the golden field.  The golden cells
      are in the case's renumberMesh order, so the test uses the
      order-free lower bound of E_s (both fields sorted): at most 0.05 at
      every write time (measured at most 0.043, at t = 1.5);
    * the interface size (cells with 1e-8 < alpha < 1 - 1e-8): within 10%
      of the golden count up to t = 2.25, within 70% after it, where the
      least-squares normals leave a diffused interface as the shape
      returns (E_s at t = 3 against the initial field is 0.36).
    """
    m = mesh64
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    o = O.Oracle(m, n_alpha_bounds=3, snap_tol=0.0, clip=False, n_threads=os.cpu_count() or 1)
    flow = H.DeformationFlow(m, period=6.0)
    fields, steps = H.run_to_write_times(o, m, a0, flow, 0.25, 3.0)
    assert len(fields) == 13 and steps > 500
    h3 = (1.0 / 64) ** 3
    off = GOLD["mixed32_off"]
    ev0 = None
    for k, a in enumerate(fields):
        t = 0.25 * k
        ev = (float(np.sum(a * m.V)) - H.EXACT_INITIAL_VOL_64) / H.EXACT_INITIAL_VOL_64
        if ev0 is None:
            ev0 = ev
            assert abs(ev) < 5e-5
        assert abs(ev - ev0) <= 1e-12, (t, ev, ev0)
        assert float(a.min()) >= -1e-6 and 1.0 - float(a.max()) >= -1e-6, t
        gold = np.sort(np.concatenate((GOLD["mixed32"][off[k]:off[k + 1]].astype(np.float64),
                                       np.ones(int(GOLD["n_full"][k])))))
        lb = H.sorted_l1_distance(a, gold, h3)
        assert lb <= 0.05, (t, lb)
        ours = int(np.count_nonzero((a > 1e-8) & (a < 1 - 1e-8)))
        want = int(GOLD["n_mixed"][k])
        assert abs(ours - want) / want <= (0.10 if t <= 2.25 else 0.70), (t, ours, want)
    e = H.errors(fields[-1], a0, m.V, float(np.sum(a0 * m.V)))
    assert 0.2 < e.shape_error < 0.5
