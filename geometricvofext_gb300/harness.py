"""Pure-advection harness: the caller side of the SimPLIC step.

Restates the reference test driver ``applications/test/plicVofAdvectionFoam``
(velocity ``updateU.H:1-70``, Courant numbers ``alphaCourantNo.H:32-55`` and
the OpenFOAM ``CourantNo.H``, time-step control ``setDeltaT.H:34-53``) and the
error metrics of ``applications/test/calcVofAdvectionErrors/updateErrors.H:1-31``.
It also builds the initial volume-fraction fields of the benchmark cases
(exact sphere overlap on uniform hexes, sub-sampled overlap elsewhere).
None of this is on the hot path; it generates the inputs the hot path consumes.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Optional, Sequence, Tuple

import numpy as np

SMALL = 1.0e-15
EXACT_INITIAL_VOL_64 = 0.0141366879746714  # calcVofAdvectionErrors.C:64


# ---------------------------------------------------------------------------
# velocity fields
# ---------------------------------------------------------------------------

def deformation_velocity(x: np.ndarray) -> np.ndarray:
    """3-D deformation field of updateU.H:13-15 (without the time factor)."""
    X, Y, Z = x[:, 0], x[:, 1], x[:, 2]
    pi = math.pi
    sx, sy, sz = np.sin(pi * X), np.sin(pi * Y), np.sin(pi * Z)
    s2x, s2y, s2z = np.sin(2 * pi * X), np.sin(2 * pi * Y), np.sin(2 * pi * Z)
    u = 2 * (sx * sx) * s2y * s2z
    v = -s2x * (sy * sy) * s2z
    w = -s2x * s2y * (sz * sz)
    return np.stack((u, v, w), axis=1)


def time_factor(t_new: float, dt: float, period: float) -> float:
    """updateU.H:59-69: mean of cos(2 pi t/T) at the end of the step and one
    step later (t is the time after ``++runTime``)."""
    if period <= 0.0:
        return 1.0
    return 0.5 * (math.cos(2.0 * math.pi * t_new / period) + math.cos(2.0 * math.pi * (t_new + dt) / period))


@dataclasses.dataclass
class Flow:
    """Per-step inputs for ``advect``: face flux, cell velocity, boundary
    velocity (``None`` = the zero fixedValue walls of the test case)."""
    phi: np.ndarray
    U: np.ndarray
    U_boundary: Optional[np.ndarray]


class DeformationFlow:
    """phi = U(Cf).Sf and U(C) from the analytic field, scaled per step by
    the period factor; walls carry fixedValue U = 0 (0.orig/U)."""

    def __init__(self, mesh, period: float = 6.0):
        self.mesh = mesh
        self.period = period
        self.U0 = deformation_velocity(mesh.C)
        Uf = deformation_velocity(mesh.Cf)
        Sf = mesh.Sf
        self.phi0 = (Uf[:, 0] * Sf[:, 0] + Uf[:, 1] * Sf[:, 1]) + Uf[:, 2] * Sf[:, 2]
        self.Ub = np.zeros((mesh.n_boundary_faces, 3))

    def at(self, t_new: float, dt: float) -> Flow:
        f = time_factor(t_new, dt, self.period)
        return Flow(self.phi0 * f, self.U0 * f, self.Ub)


class TranslationFlow:
    """Uniform velocity (the translation test: U = (0.5, 0.5, 0.5))."""

    def __init__(self, mesh, U=(0.5, 0.5, 0.5)):
        self.mesh = mesh
        u = np.asarray(U, dtype=np.float64)
        self.U0 = np.broadcast_to(u, (mesh.n_cells, 3)).copy()
        Sf = mesh.Sf
        self.phi0 = (u[0] * Sf[:, 0] + u[1] * Sf[:, 1]) + u[2] * Sf[:, 2]
        self.Ub = np.broadcast_to(u, (mesh.n_boundary_faces, 3)).copy()

    def at(self, t_new: float, dt: float) -> Flow:
        return Flow(self.phi0, self.U0, self.Ub)


# ---------------------------------------------------------------------------
# Courant numbers and time-step control
# ---------------------------------------------------------------------------

def surface_sum_mag(mesh, phi: np.ndarray) -> np.ndarray:
    """fvc::surfaceSum(mag(phi)) on cells (internal + boundary faces)."""
    s = np.zeros(mesh.n_cells)
    a = np.abs(phi)
    nfi = mesh.n_internal_faces
    np.add.at(s, mesh.owner, a)
    np.add.at(s, mesh.neighbour, a[:nfi])
    return s


def courant_numbers(mesh, phi: np.ndarray, alpha: np.ndarray, dt: float) -> Tuple[float, float]:
    """(CoNum, alphaCoNum) of OpenFOAM CourantNo.H and alphaCourantNo.H:40-52;
    the interface number counts cells with 0.01 <= alpha <= 0.99."""
    sumPhi = surface_sum_mag(mesh, phi)
    co = 0.5 * float(np.max(sumPhi / mesh.V)) * dt
    mask = (alpha - 0.01 >= 0) & (0.99 - alpha >= 0)
    aco = 0.5 * float(np.max(np.where(mask, sumPhi, 0.0) / mesh.V)) * dt
    return co, aco


def next_delta_t(dt: float, co: float, aco: float, maxCo: float = 0.5, maxAlphaCo: float = 0.5,
                 maxDeltaT: float = 0.2) -> float:
    """setDeltaT.H:34-53."""
    maxDeltaTFact = min(maxCo / (co + SMALL), maxAlphaCo / (aco + SMALL))
    deltaTFact = min(min(maxDeltaTFact, 1.0 + 0.1 * maxDeltaTFact), 1.2)
    return min(deltaTFact * dt, maxDeltaT)


def cfl_delta_t(mesh, phi_full_speed: np.ndarray, co: float = 0.5) -> float:
    """Fixed time step that puts the full-speed field at Courant number
    ``co`` on every cell (the bound the adaptive control converges to)."""
    sumPhi = surface_sum_mag(mesh, phi_full_speed)
    return co / (0.5 * float(np.max(sumPhi / mesh.V)))


# ---------------------------------------------------------------------------
# initial volume fractions
# ---------------------------------------------------------------------------

def _disk_corner_area(r, a, b):
    """Area of {u^2 + v^2 <= r^2, u <= a, v <= b} (closed form)."""
    r = np.maximum(r, 0.0)
    a = np.clip(a, -r, r)
    bb = np.clip(b, -r, r)
    w = np.sqrt(np.maximum(r * r - bb * bb, 0.0))

    def S(u):  # primitive of sqrt(r^2 - u^2)
        uu = np.clip(u, -r, r)
        s = np.sqrt(np.maximum(r * r - uu * uu, 0.0))
        return 0.5 * (uu * s + r * r * np.arcsin(np.where(r > 0, uu / np.where(r > 0, r, 1.0), 0.0)))

    def seg_inner(u0, u1):  # integral of (b + s(u)) over [u0, u1] with |u| < w
        u1 = np.maximum(u0, u1)
        return bb * (u1 - u0) + S(u1) - S(u0)

    def seg_outer(u0, u1):  # integral of 2 s(u) (b >= 0) or 0 (b < 0)
        u1 = np.maximum(u0, u1)
        return np.where(bb >= 0, 2.0 * (S(u1) - S(u0)), 0.0)

    # pieces of [-r, a]: [-r, -w] outer, [-w, w] inner, [w, r] outer
    p1 = seg_outer(-r, np.minimum(a, -w))
    p2 = seg_inner(np.minimum(np.maximum(-w, -r), a), np.minimum(w, a))
    p3 = seg_outer(np.minimum(w, a), a)
    return np.where(r > 0, p1 + p2 + p3, 0.0)


def _sphere_box_volume(lo, hi, centre, R, G=16):
    """Volume of a sphere inside axis-aligned boxes: the (y, z) cross-section
    area of each x-slice is exact (disk-rectangle inclusion-exclusion), and
    x is integrated by Gauss-Legendre on the pieces between the kinks where
    the slice radius meets a box edge or corner."""
    c = np.asarray(centre, float)
    nb = lo.shape[0]
    dy = np.stack((lo[:, 1] - c[1], hi[:, 1] - c[1]), axis=1)
    dz = np.stack((lo[:, 2] - c[2], hi[:, 2] - c[2]), axis=1)
    rho = [np.abs(dy[:, 0]), np.abs(dy[:, 1]), np.abs(dz[:, 0]), np.abs(dz[:, 1])]
    for i in range(2):
        for j in range(2):
            rho.append(np.sqrt(dy[:, i] ** 2 + dz[:, j] ** 2))
    kinks = [np.full(nb, c[0] - R), np.full(nb, c[0] + R)]
    for p in rho:
        h = np.sqrt(np.maximum(R * R - p * p, 0.0))
        kinks += [c[0] - h, c[0] + h]
    K = np.stack([lo[:, 0], hi[:, 0]] + [np.clip(k, lo[:, 0], hi[:, 0]) for k in kinks], axis=1)
    K.sort(axis=1)
    xg, wg = np.polynomial.legendre.leggauss(G)
    vol = np.zeros(nb)
    for p in range(K.shape[1] - 1):
        x0, x1 = K[:, p], K[:, p + 1]
        half = 0.5 * (x1 - x0)
        mid = 0.5 * (x0 + x1)
        for g in range(G):
            x = mid + half * xg[g]
            r = np.sqrt(np.maximum(R * R - (x - c[0]) ** 2, 0.0))
            A = (_disk_corner_area(r, dy[:, 1], dz[:, 1]) - _disk_corner_area(r, dy[:, 0], dz[:, 1])
                 - _disk_corner_area(r, dy[:, 1], dz[:, 0]) + _disk_corner_area(r, dy[:, 0], dz[:, 0]))
            vol += (half * wg[g]) * A
    return vol


def _chord_overlap(lo, hi, centre, R):
    return _sphere_box_volume(lo, hi, centre, R)


def _cell_boxes(mesh):
    """Axis-aligned bounding box of every cell."""
    if mesh.face_size() > 0:
        offs, cf = mesh.cell_faces()
        fp = mesh.faces_dense()
        nc = mesh.n_cells
        k = int(offs[1] - offs[0])
        faces = cf.reshape(nc, k)
        pts = mesh.points[fp[faces].reshape(nc, -1)]
        return pts.min(axis=1), pts.max(axis=1)
    # any face sizes: fold every face's points into its owner and neighbour
    fo = mesh.face_offsets.astype(np.int64)
    face_of = np.repeat(np.arange(mesh.n_faces), np.diff(fo))
    P = mesh.points[mesh.face_points]
    lo = np.full((mesh.n_cells, 3), np.inf)
    hi = np.full((mesh.n_cells, 3), -np.inf)
    for cells in (mesh.owner[face_of], None):
        if cells is None:
            inner = face_of < mesh.n_internal_faces
            cells, Q = mesh.neighbour[face_of[inner]], P[inner]
        else:
            Q = P
        for k in range(3):
            np.minimum.at(lo[:, k], cells, Q[:, k])
            np.maximum.at(hi[:, k], cells, Q[:, k])
    return lo, hi


def sphere_alpha(mesh, centre: Sequence[float], R: float) -> np.ndarray:
    """Volume fraction of a sphere.  Uniform hex blocks use the exact chord
    integration; other meshes sub-sample each interface cell (tets of the
    cell centre and face fans, 6^3 barycentric points each)."""
    c = np.asarray(centre, dtype=np.float64)
    lo, hi = _cell_boxes(mesh)
    near = np.clip(c, lo, hi)
    dnear = np.sqrt(((near - c) ** 2).sum(axis=1))
    far = np.maximum(np.abs(lo - c), np.abs(hi - c))
    dfar = np.sqrt((far ** 2).sum(axis=1))
    alpha = np.zeros(mesh.n_cells)
    alpha[dfar <= R] = 1.0
    band = np.flatnonzero((dnear < R) & (dfar > R))
    if band.size == 0:
        return alpha
    if mesh.kind in ("hex", "hex-refined"):  # axis-aligned box cells
        v = _chord_overlap(lo[band], hi[band], c, R)
        alpha[band] = np.clip(v / mesh.V[band], 0.0, 1.0)
    else:
        alpha[band] = _sampled_fraction(mesh, band, lambda x: ((x - c) ** 2).sum(axis=-1) <= R * R)
    return alpha


def _sampled_fraction(mesh, cells, inside, m=6):
    """Volume-weighted fraction of sample points inside, over the tets
    (cell centre, face centre, edge) of each cell."""
    offs, cf = mesh.cell_faces()
    fp = mesh.faces_dense()
    n = fp.shape[1]
    # barycentric lattice of m^3 interior points per tet (midpoint rule)
    g = (np.arange(m) + 0.5) / m
    u, v, w = np.meshgrid(g, g, g, indexing="ij")
    u, v, w = u.ravel(), v.ravel(), w.ravel()
    # map unit cube to tet via the Duffy-like collapse (weights = jacobian)
    b1 = u
    b2 = v * (1 - u)
    b3 = w * (1 - u) * (1 - v)
    jac = (1 - u) ** 2 * (1 - v)
    out = np.zeros(cells.size)
    k = int(offs[1] - offs[0])
    faces = cf.reshape(mesh.n_cells, k)[cells]
    C = mesh.C[cells]
    tot = np.zeros(cells.size)
    for j in range(k):
        f = faces[:, j]
        Cf = mesh.Cf[f]
        for e in range(n):
            p0 = mesh.points[fp[f, e]]
            p1 = mesh.points[fp[f, (e + 1) % n]]
            e1, e2, e3 = Cf - C, p0 - C, p1 - C
            det = np.abs((e1[:, 0] * (e2[:, 1] * e3[:, 2] - e2[:, 2] * e3[:, 1])
                          - e1[:, 1] * (e2[:, 0] * e3[:, 2] - e2[:, 2] * e3[:, 0])
                          + e1[:, 2] * (e2[:, 0] * e3[:, 1] - e2[:, 1] * e3[:, 0])))
            x = (C[:, None, :] + b1[None, :, None] * e1[:, None, :] + b2[None, :, None] * e2[:, None, :]
                 + b3[None, :, None] * e3[:, None, :])
            ins = inside(x).astype(np.float64)
            out += det * (ins * jac[None, :]).sum(axis=1)
            tot += det * jac.sum()
    return np.clip(out / tot, 0.0, 1.0)


def spheres_and_slab_alpha(mesh, n_spheres: int = 200, rmin: float = 0.01, rmax: float = 0.04,
                           slab_z: float = 0.2, seed: int = 2024) -> np.ndarray:
    """Seeded union of non-overlapping spheres plus the slab z < slab_z
    (the 320^3 scale case); spheres keep a 2h gap from each other and
    from the slab so their fractions add."""
    rng = np.random.default_rng(seed)
    h = mesh.h
    cs, rs = [], []
    tries = 0
    while len(cs) < n_spheres and tries < 100000:
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(r + 2 * h, 1 - r - 2 * h, size=3)
        if c[2] - r < slab_z + 2 * h:
            continue
        if any(np.linalg.norm(c - c2) < r + r2 + 2 * h for c2, r2 in zip(cs, rs)):
            continue
        cs.append(c)
        rs.append(r)
    alpha = np.zeros(mesh.n_cells)
    lo, hi = _cell_boxes(mesh)
    # slab: exact on hexes aligned with z
    alpha += np.clip((np.minimum(hi[:, 2], slab_z) - lo[:, 2]) / (hi[:, 2] - lo[:, 2]), 0.0, 1.0)
    for c, r in zip(cs, rs):
        alpha += sphere_alpha_box(mesh, lo, hi, c, r)
    return np.clip(alpha, 0.0, 1.0)


def sphere_alpha_box(mesh, lo, hi, c, R):
    c = np.asarray(c)
    near = np.clip(c, lo, hi)
    dnear = np.sqrt(((near - c) ** 2).sum(axis=1))
    far = np.maximum(np.abs(lo - c), np.abs(hi - c))
    dfar = np.sqrt((far ** 2).sum(axis=1))
    out = np.zeros(mesh.n_cells)
    out[dfar <= R] = 1.0
    band = np.flatnonzero((dnear < R) & (dfar > R))
    if band.size:
        out[band] = np.clip(_chord_overlap(lo[band], hi[band], c, R) / mesh.V[band], 0.0, 1.0)
    return out


# ---------------------------------------------------------------------------
# error metrics (updateErrors.H:9-31; E_p needs iso-surface cutting and is
# not restated)
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Errors:
    volume_error: float       # E_v
    min_alpha: float
    one_minus_max_alpha: float
    shape_error: float        # E_s
    boundedness: float        # max(-min alpha, max alpha - 1, 0)


def errors(alpha: np.ndarray, alpha_ref: np.ndarray, V: np.ndarray, vol0: float) -> Errors:
    vol = float(np.sum(alpha * V))
    ev = (vol - vol0) / vol0
    es = float(np.sum(np.abs(alpha - alpha_ref) * V) / np.sum(alpha_ref * V))
    mn, mx = float(alpha.min()), float(alpha.max())
    return Errors(ev, mn, 1.0 - mx, es, max(-mn, mx - 1.0, 0.0))


# ---------------------------------------------------------------------------
# a driver in the reference's shape (plicVof.H:13-54)
# ---------------------------------------------------------------------------

def run_adaptive(solver, mesh, alpha0, flow, t_end, dt0=1e-3, maxCo=0.5, maxAlphaCo=0.5,
                 maxDeltaT=0.2, max_steps=None, callback=None):
    """Advance ``solver`` (anything with reconstruct(alpha) and
    advect(alpha, phi, U, dt, U_boundary=...)) from t=0 to t_end with the
    reference's adaptive time step.  Returns (alpha, t, steps)."""
    alpha = np.array(alpha0, dtype=np.float64, copy=True)
    t = 0.0
    dt = dt0
    phi = np.zeros(mesh.n_faces)  # initial U = 0 (0.orig/U)
    co, _ = courant_numbers(mesh, phi, alpha, dt)
    dt = min(maxCo * dt / (co + SMALL), min(dt, maxDeltaT))  # setInitialDeltaT
    steps = 0
    while t < t_end - 1e-12 and (max_steps is None or steps < max_steps):
        co, aco = courant_numbers(mesh, phi, alpha, dt)
        dt = next_delta_t(dt, co, aco, maxCo, maxAlphaCo, maxDeltaT)
        if t + dt > t_end:
            dt = t_end - t
        t += dt
        fl = flow.at(t, dt)
        phi = fl.phi
        solver.reconstruct(alpha)
        alpha = solver.advect(alpha, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        steps += 1
        if callback is not None:
            callback(steps, t, dt, alpha)
    return alpha, t, steps


def run_to_write_times(solver, mesh, alpha0, flow, write_interval, t_end, dt0=1e-3, maxCo=0.5,
                       maxAlphaCo=0.5, maxDeltaT=0.2):
    """The reference test's time loop (controlDict: adjustTimeStep yes,
    writeControl adjustableRunTime): the Courant-limited step of
    setDeltaT.H, then spread evenly over the steps left to the next write
    time (rounded up), changed by at most x2 / x0.2 per step, so every
    multiple of ``write_interval`` is hit exactly.  Returns the fields at
    the write times (t = 0 included) and the number of steps."""
    alpha = np.array(alpha0, dtype=np.float64, copy=True)
    out = [alpha.copy()]
    t = 0.0
    dt = dt0
    phi = np.zeros(mesh.n_faces)
    co, _ = courant_numbers(mesh, phi, alpha, dt)
    dt = min(maxCo * dt / (co + SMALL), min(dt, maxDeltaT))
    steps = 0
    n_writes = int(round(t_end / write_interval))
    for w in range(1, n_writes + 1):
        t_write = w * write_interval
        while t < t_write - 1e-12:
            co, aco = courant_numbers(mesh, phi, alpha, dt)
            dt = next_delta_t(dt, co, aco, maxCo, maxAlphaCo, maxDeltaT)
            to_write = max(0.0, t_write - t)
            n_left = max(1, int(math.ceil(to_write / dt - 1e-9)))
            new_dt = to_write / n_left
            dt = min(new_dt, 2.0 * dt) if new_dt >= dt else max(new_dt, 0.2 * dt)
            t = t_write if n_left == 1 else t + dt
            fl = flow.at(t, dt)
            phi = fl.phi
            solver.reconstruct(alpha)
            alpha = solver.advect(alpha, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
            steps += 1
        out.append(alpha.copy())
    return out, steps


def sorted_l1_distance(alpha: np.ndarray, ref_sorted_nonzero: np.ndarray, V: float) -> float:
    """sum |a_i - b_pi(i)| V over the best cell correspondence pi (both
    fields sorted, zeros padding the shorter list) divided by sum(b) V, on a
    mesh of equal cell volumes V: a lower bound of the shape error E_s
    (updateErrors.H:31) that needs no cell order, because in one dimension
    the monotone matching minimises the sum of |a - b|."""
    a = np.sort(alpha[alpha != 0.0])
    b = np.asarray(ref_sorted_nonzero, dtype=np.float64)
    n = max(a.size, b.size)
    a = np.concatenate((np.zeros(n - a.size), a))
    b = np.concatenate((np.zeros(n - b.size), b))
    return float(np.sum(np.abs(a - b)) * V / (np.sum(b) * V))
