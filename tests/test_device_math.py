"""Host-side checks of device helpers that compile for both sides (built
with nvcc, run on the CPU): the lattice face-slot formula the update uses
for interior cells, and the FP32 cube fractions of the learned form's
fallback test."""

import os
import subprocess

import numpy as np
import pytest

from geometricvofext_gb300 import build as B, meshgen as mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("devmath") / "device_math_check")
    src = os.path.join(ROOT, "tests", "cpp", "device_math_check.cu")
    cmd = [B.nvcc(), *B.ARCH, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "geometricvofext_gb300", "csrc"),
           "-I", os.path.join(ROOT, "include"), src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _slot_records(mesh):
    """Per cell, the faces in ascending id with the cell across and the
    neighbour-side bit (the layout of the update's face-slot records)."""
    own, nei, nfi = mesh.owner, mesh.neighbour, mesh.n_internal_faces
    rec = [[] for _ in range(mesh.n_cells)]
    for f in range(mesh.n_faces):
        o = int(own[f])
        rec[o].append((int(nei[f]) if f < nfi else -1, f))
        if f < nfi:
            rec[int(nei[f])].append((o, f | (1 << 31)))
    return [sorted(r, key=lambda t: t[1] & 0x7FFFFFFF) for r in rec]


@pytest.mark.parametrize("n", [3, 5, 7])
def test_lattice_slots_match_the_mesh(checker, n):
    mesh = mg.make_mesh("hex", n)
    rec = _slot_records(mesh)
    out = subprocess.run([checker, "slots", str(n), str(n), str(n)], capture_output=True, text=True, check=True)
    lines = out.stdout.split("\n")[:-1]
    interior = [c for c in range(mesh.n_cells)
                if 0 < c % n < n - 1 and 0 < (c // n) % n < n - 1 and 0 < c // (n * n) < n - 1]
    assert len(lines) == len(interior)
    for line in lines:
        v = [int(x) for x in line.split()]
        c = v[0]
        got = [(v[1 + 2 * q], v[2 + 2 * q] & 0xFFFFFFFF) for q in range(6)]
        want = [(x, y & 0xFFFFFFFF) for x, y in rec[c]]
        assert got == want, (c, got, want)


def _cube_fraction(a, m):
    """Inclusion-exclusion over the cube corners (float64)."""
    if a <= 0.0:
        return 0.0
    if a >= 1.0:
        return 1.0
    tot = 0.0
    for i in (0, 1):
        for j in (0, 1):
            for k in (0, 1):
                t = a - (i * m[0] + j * m[1] + k * m[2])
                if t > 0:
                    tot += (-1) ** (i + j + k) * t ** 3
    return tot / (6.0 * m[0] * m[1] * m[2])


def test_cube_fractions_and_inverse(checker):
    out = subprocess.run([checker, "cube"], capture_output=True, text=True, check=True)
    rows = np.array([[float(x) for x in line.split()] for line in out.stdout.split("\n")[:-1]])
    assert rows.shape[0] == 6 * 41
    for m1, m2, m3, a, F, dF, inv in rows:
        m = (m1, m2, m3)
        assert abs(m1 + m2 + m3 - 1.0) < 1e-6 and m1 <= m2 <= m3
        assert abs(F - _cube_fraction(a, m)) < 2e-5, (m, a, F)
        if 0.0 < a < 1.0:
            h = 1e-4
            num = (_cube_fraction(a + h, m) - _cube_fraction(a - h, m)) / (2 * h)
            assert abs(dF - num) < 2e-2 * max(1.0, num), (m, a, dF, num)
        if 1e-4 < F < 1 - 1e-4:
            assert abs(_cube_fraction(inv, m) - F) < 2e-5, (m, F, inv)


def test_fast_division_by_invariant_divisors(checker):
    """fastDivide (multiply-high and shifts, the lattice position of a cell
    in the update) equals the integer division for every divisor 2..4096
    and the lattice layer sizes, over random numerators, numerators next to
    multiples of the divisor and the 31- and 32-bit edges."""
    r = subprocess.run([checker, "fdiv", "4000000", "9"], capture_output=True, text=True, check=True)
    n, bad = map(int, r.stdout.split())
    assert n > 4000000 and bad == 0


def test_quotient_of_a_product_is_correctly_rounded(checker):
    """dv / dt for dv = RN(x dt) from x with one Newton correction
    (divOfProduct) equals IEEE division bit for bit: x and dt random over
    wide exponent ranges, powers of two and all-ones significands (host
    instantiation; the device one runs in the GPU test below)."""
    r = subprocess.run([checker, "qprod", "20000000", "5"], capture_output=True, text=True, check=True)
    n, bad = map(int, r.stdout.split())
    assert n == 20000000 and bad == 0


def test_division_by_reciprocal_is_correctly_rounded(checker):
    """The update's division a / b through the correctly rounded reciprocal
    and two FMA Newton corrections (divByRecip) equals IEEE division bit for
    bit, over random operands of the whole exponent range and near the
    edges of its fast range (built with nvcc for the host, run on the CPU;
    the same test of the device instantiation runs on the GPU)."""
    r = subprocess.run([checker, "div", "20000000", "1"], capture_output=True, text=True, check=True)
    n, bad = map(int, r.stdout.split())
    assert n == 20000000 and bad == 0


@pytest.mark.gpu
def test_division_by_reciprocal_on_the_gpu(tmp_path):
    """The device instantiations of divByRecip and divOfProduct against
    CUDA's own double division, 2^28 samples each on the GPU: no mismatch."""
    out = str(tmp_path / "div_gpu_check")
    src = os.path.join(ROOT, "tests", "cpp", "div_gpu_check.cu")
    cmd = [B.nvcc(), *B.ARCH, "-O2", "-std=c++17", "-fmad=false", "-I",
           os.path.join(ROOT, "geometricvofext_gb300", "csrc"), src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([out, str(1 << 28)], capture_output=True, text=True, check=True, timeout=300)
    n, bad = map(int, r.stdout.split())
    assert n == 1 << 28 and bad == 0
    # the quotient of a product from the product (divOfProduct)
    r = subprocess.run([out, str(1 << 28), "prod"], capture_output=True, text=True, check=True, timeout=300)
    n, bad = map(int, r.stdout.split())
    assert n == 1 << 28 and bad == 0


def test_plane_angle_matches_the_oracle_and_atan2(checker):
    """planeAngle, the atan2 that orders the PLIC polygon points on the GPU
    (correctly rounded operations only), built for the host: bit for bit the
    oracle's copy, and within 8 ulp of the C library's atan2 (random pairs
    over magnitudes 2^-12 .. 2^16 and all four quadrants)."""
    import math
    import struct

    from oracle import oracle as O

    r = subprocess.run([checker, "angle", "20000", "7"], capture_output=True, text=True, check=True)
    f = lambda h: struct.unpack("<d", struct.pack("<Q", int(h, 16)))[0]  # noqa: E731
    worst = 0.0
    for line in r.stdout.split("\n"):
        if not line:
            continue
        y, x, a = map(f, line.split())
        assert struct.pack("<d", O.plane_angle(y, x)) == struct.pack("<d", a), (y, x)
        ref = math.atan2(y, x)
        worst = max(worst, abs(a - ref) / math.ulp(ref))
    assert worst <= 8.0, worst


def test_plane_angle_special_values():
    """Signed zeros, infinities and NaN as C's atan2 has them."""
    import math

    from oracle import oracle as O

    inf = math.inf
    for y in (0.0, -0.0, 1.0, -1.0, inf, -inf, 3e-300, -2.5e300):
        for x in (0.0, -0.0, 1.0, -1.0, inf, -inf, 7e-310, -4e299):
            a, ref = O.plane_angle(y, x), math.atan2(y, x)
            assert math.copysign(1.0, a) == math.copysign(1.0, ref), (y, x, a, ref)
            assert abs(a - ref) <= 4 * math.ulp(ref), (y, x, a, ref)
    assert math.isnan(O.plane_angle(math.nan, 1.0)) and math.isnan(O.plane_angle(1.0, math.nan))
