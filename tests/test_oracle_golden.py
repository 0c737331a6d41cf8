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


def test_golden_mixed_counts_follow_the_flow(mesh64):
    """Advance the oracle with the reference test's settings (64^3, T=6,
    CFL 0.5, nAlphaBounds 3, clip off) to t=0.5 and compare the interface
    size and value distribution with the golden field at t=0.5."""
    m = mesh64
    a0 = H.sphere_alpha(m, (0.35, 0.35, 0.35), 0.15)
    o = O.Oracle(m, n_alpha_bounds=3, snap_tol=0.0, clip=False, n_threads=os.cpu_count() or 1)
    flow = H.DeformationFlow(m, period=6.0)
    a, t, steps = H.run_adaptive(o, m, a0, flow, t_end=0.5)
    assert abs(t - 0.5) < 1e-12
    vol0 = float(np.sum(a0 * m.V))
    assert abs(float(np.sum(a * m.V)) - vol0) / vol0 < 1e-12
    tol = 1e-3
    ours = int(np.count_nonzero((a > tol) & (a < 1 - tol)))
    gold = int(GOLD["n_mixed"][2])
    # interface cell count within 15% of the exact solution's
    assert abs(ours - gold) / gold < 0.15, (ours, gold)
