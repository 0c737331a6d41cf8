"""Synthetic polyMesh generators and OpenFOAM-style mesh metrics (numpy).

The SimPLIC hot path consumes an OpenFOAM ``polyMesh``: points, faces as point
lists whose right-hand normal points out of the owner cell, ``owner`` /
``neighbour`` with internal faces first in upper-triangular order, boundary
faces grouped by patch.  These generators build such meshes for the workloads
the reference tests on:

* uniform hex blocks (``blockMesh`` of
  ``tutorials/test/plicVofAdvectionFoam/system/blockMeshDict:17-92``: one
  ``hex (0 1 2 3 4 5 6 7)`` block, patches top/left/back/right/bottom/front);
* the same block with interior points jittered (non-planar faces);
* every hex split into 6 tetrahedra (Kuhn split along the main diagonal).

Mesh metrics follow the OpenFOAM primitiveMesh algorithms the reference relies
on (``mesh.Cf()``, ``mesh.Sf()``, ``mesh.C()``, ``mesh.V()``): face centre and
area by a triangle fan about the point average -- the same algorithm as
``cutFace::calcSubFaceCentreAndArea`` (``src/SimPLIC/cut/cutFace/cutFace.C:37-96``)
-- and cell centre and volume by face pyramids about the average of the face
centres, accumulated over owned faces then neighbour faces (the ``cells()``
order).  Every floating-point operation is written out in a fixed order so the
arrays are identical on every machine (numpy ufuncs never contract a*b+c).
"""

from __future__ import annotations

import dataclasses
from typing import List, Optional, Tuple

import numpy as np

ROOTVSMALL = 1.0e-150
VSMALL = 1.0e-300

# Patch order and the hex-model face used for each patch, as in the
# reference test case blockMeshDict (top, left, back, right, bottom, front).
_PATCHES = ("top", "left", "back", "right", "bottom", "front")


@dataclasses.dataclass
class PolyMesh:
    points: np.ndarray          # (Np, 3) float64
    face_offsets: np.ndarray    # (Nf+1,) int32
    face_points: np.ndarray     # (sum,) int32
    owner: np.ndarray           # (Nf,) int32
    neighbour: np.ndarray       # (Nfi,) int32
    n_cells: int
    patches: List[Tuple[str, int, int]]  # (name, start, size)
    kind: str = "hex"
    # metrics (filled by compute_metrics)
    C: Optional[np.ndarray] = None      # (Nc, 3)
    V: Optional[np.ndarray] = None      # (Nc,)
    Cf: Optional[np.ndarray] = None     # (Nf, 3)
    Sf: Optional[np.ndarray] = None     # (Nf, 3)
    magSf: Optional[np.ndarray] = None  # (Nf,)
    h: float = 0.0                      # nominal spacing

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def n_internal_faces(self) -> int:
        return int(self.neighbour.shape[0])

    @property
    def n_boundary_faces(self) -> int:
        return self.n_faces - self.n_internal_faces

    def face_size(self) -> int:
        """Points per face when all faces have the same size, else -1."""
        d = np.diff(self.face_offsets)
        return int(d[0]) if d.size and np.all(d == d[0]) else -1

    def faces_dense(self) -> np.ndarray:
        n = self.face_size()
        assert n > 0, "faces_dense needs uniform face size"
        return self.face_points.reshape(-1, n)

    def cell_faces(self) -> Tuple[np.ndarray, np.ndarray]:
        """OpenFOAM ``primitiveMesh::cells()`` as CSR: for each cell its owned
        faces in ascending face order, then the faces it neighbours in
        ascending order.  Returns (offsets[Nc+1], faces)."""
        nc = self.n_cells
        own = self.owner.astype(np.int64)
        nei = self.neighbour.astype(np.int64)
        n_own = np.bincount(own, minlength=nc)
        n_nei = np.bincount(nei, minlength=nc)
        counts = n_own + n_nei
        offs = np.zeros(nc + 1, dtype=np.int64)
        np.cumsum(counts, out=offs[1:])
        out = np.empty(int(offs[-1]), dtype=np.int32)
        o_order = np.argsort(own, kind="stable")
        o_start = np.zeros(nc + 1, dtype=np.int64)
        np.cumsum(n_own, out=o_start[1:])
        rank_o = np.arange(own.size, dtype=np.int64) - o_start[own[o_order]]
        out[offs[own[o_order]] + rank_o] = o_order
        n_order = np.argsort(nei, kind="stable")
        n_start = np.zeros(nc + 1, dtype=np.int64)
        np.cumsum(n_nei, out=n_start[1:])
        rank_n = np.arange(nei.size, dtype=np.int64) - n_start[nei[n_order]]
        out[offs[nei[n_order]] + n_own[nei[n_order]] + rank_n] = n_order
        return offs.astype(np.int64), out


# ---------------------------------------------------------------------------
# vector helpers with a fixed operation order
# ---------------------------------------------------------------------------

def _cross(a, b):
    return np.stack(
        (
            a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
            a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
            a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0],
        ),
        axis=1,
    )


def _dot(a, b):
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def _mag(a):
    return np.sqrt((a[:, 0] * a[:, 0] + a[:, 1] * a[:, 1]) + a[:, 2] * a[:, 2])


# ---------------------------------------------------------------------------
# metrics
# ---------------------------------------------------------------------------

def face_centres_areas(points: np.ndarray, faces: np.ndarray, chunk: int = 1 << 18):
    """Face centres and area vectors for faces of uniform size.

    Triangles use the direct formula; larger faces the triangle fan about the
    point average (the algorithm of ``cutFace.C:37-96``)."""
    nf, n = faces.shape
    Cf = np.empty((nf, 3))
    Sf = np.empty((nf, 3))
    for s in range(0, nf, chunk):
        e = min(nf, s + chunk)
        P = [points[faces[s:e, i]] for i in range(n)]
        if n == 3:
            Cf[s:e] = (1.0 / 3.0) * ((P[0] + P[1]) + P[2])
            Sf[s:e] = 0.5 * _cross(P[1] - P[0], P[2] - P[0])
            continue
        fc = P[0].copy()
        for i in range(1, n):
            fc += P[i]
        fc /= float(n)
        sumN = np.zeros((e - s, 3))
        sumA = np.zeros(e - s)
        sumAc = np.zeros((e - s, 3))
        for i in range(n):
            this = P[i]
            nxt = P[(i + 1) % n]
            c = (this + nxt) + fc
            nv = _cross(nxt - this, fc - this)
            a = _mag(nv)
            sumN += nv
            sumA += a
            sumAc += a[:, None] * c
        small = sumA < ROOTVSMALL
        cf = ((1.0 / 3.0) * sumAc) / np.where(small, 1.0, sumA)[:, None]
        sf = 0.5 * sumN
        cf[small] = fc[small]
        sf[small] = 0.0
        Cf[s:e] = cf
        Sf[s:e] = sf
    return Cf, Sf


def cell_centres_volumes(mesh: PolyMesh, Cf: np.ndarray, Sf: np.ndarray, chunk: int = 1 << 18):
    """Cell centres and volumes (pyramids about the face-centre average),
    accumulated over owned faces then neighbour faces in face order."""
    offs, cf = mesh.cell_faces()
    nc = mesh.n_cells
    cnt = np.diff(offs)
    assert np.all(cnt == cnt[0]), "uniform cell valence expected"
    k = int(cnt[0])
    table = cf.reshape(nc, k)
    own = mesh.owner
    C = np.empty((nc, 3))
    V = np.empty(nc)
    for s in range(0, nc, chunk):
        e = min(nc, s + chunk)
        tb = table[s:e].astype(np.int64)
        cEst = np.zeros((e - s, 3))
        for j in range(k):
            cEst += Cf[tb[:, j]]
        cEst /= float(k)
        Cc = np.zeros((e - s, 3))
        Vc = np.zeros(e - s)
        cells = np.arange(s, e)
        for j in range(k):
            f = tb[:, j]
            is_own = own[f] == cells
            cfj = Cf[f]
            d = np.where(is_own[:, None], cfj - cEst, cEst - cfj)
            pyr3 = _dot(Sf[f], d)
            pc = 0.75 * cfj + 0.25 * cEst
            Cc += pyr3[:, None] * pc
            Vc += pyr3
        ok = np.abs(Vc) > VSMALL
        C[s:e] = np.where(ok[:, None], Cc / np.where(ok, Vc, 1.0)[:, None], cEst)
        V[s:e] = Vc * (1.0 / 3.0)
    return C, V


def compute_metrics(mesh: PolyMesh) -> PolyMesh:
    faces = mesh.faces_dense()
    Cf, Sf = face_centres_areas(mesh.points, faces)
    mesh.Cf, mesh.Sf = Cf, Sf
    mesh.magSf = _mag(Sf)
    mesh.C, mesh.V = cell_centres_volumes(mesh, Cf, Sf)
    return mesh


# ---------------------------------------------------------------------------
# generators
# ---------------------------------------------------------------------------

def hex_mesh(n: int, length: float = 1.0, jitter: float = 0.0, seed: int = 12345,
             metrics: bool = True) -> PolyMesh:
    """Uniform ``n^3`` hex block on ``[0, length]^3`` (blockMesh numbering:
    point ``i + (n+1)(j + (n+1)k)``, cell ``i + n(j + n k)``).

    ``jitter`` > 0 moves every interior point by an independent uniform
    offset in ``[-jitter*h, +jitter*h]`` per coordinate (seeded); boundary
    points stay on the block faces, so faces become non-planar."""
    n1 = n + 1
    h = length / n
    ii = np.arange(n1, dtype=np.float64)
    coord = ii * length / n
    coord[-1] = length
    k, j, i = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    pts = np.stack((coord[i.ravel()], coord[j.ravel()], coord[k.ravel()]), axis=1)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        off = rng.uniform(-jitter * h, jitter * h, size=pts.shape)
        interior = ((i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)).ravel()
        pts[interior] += off[interior]

    def pid(i, j, k):
        return (i + n1 * (j + n1 * k)).astype(np.int32)

    nc = n * n * n
    c = np.arange(nc, dtype=np.int64)
    ci = c % n
    cj = (c // n) % n
    ck = c // (n * n)
    # internal faces, upper-triangular: per owner the +x, +y, +z faces
    valid = np.stack((ci < n - 1, cj < n - 1, ck < n - 1), axis=1)
    own_c, d = np.nonzero(valid)
    oi, oj, ok = ci[own_c], cj[own_c], ck[own_c]
    fp = np.empty((own_c.size, 4), dtype=np.int32)
    nb = np.empty(own_c.size, dtype=np.int64)
    m = d == 0  # +x face (hex face 1 2 6 5)
    fp[m] = np.stack((pid(oi[m] + 1, oj[m], ok[m]), pid(oi[m] + 1, oj[m] + 1, ok[m]),
                      pid(oi[m] + 1, oj[m] + 1, ok[m] + 1), pid(oi[m] + 1, oj[m], ok[m] + 1)), axis=1)
    nb[m] = own_c[m] + 1
    m = d == 1  # +y face (hex face 3 7 6 2)
    fp[m] = np.stack((pid(oi[m], oj[m] + 1, ok[m]), pid(oi[m], oj[m] + 1, ok[m] + 1),
                      pid(oi[m] + 1, oj[m] + 1, ok[m] + 1), pid(oi[m] + 1, oj[m] + 1, ok[m])), axis=1)
    nb[m] = own_c[m] + n
    m = d == 2  # +z face (hex face 4 5 6 7)
    fp[m] = np.stack((pid(oi[m], oj[m], ok[m] + 1), pid(oi[m] + 1, oj[m], ok[m] + 1),
                      pid(oi[m] + 1, oj[m] + 1, ok[m] + 1), pid(oi[m], oj[m] + 1, ok[m] + 1)), axis=1)
    nb[m] = own_c[m] + n * n
    owner = [own_c.astype(np.int32)]
    faces = [fp]
    patches = []
    start = own_c.size
    for name in _PATCHES:
        if name == "top":
            sel = ck == n - 1
        elif name == "bottom":
            sel = ck == 0
        elif name == "left":
            sel = cj == 0
        elif name == "right":
            sel = cj == n - 1
        elif name == "back":
            sel = ci == 0
        else:
            sel = ci == n - 1
        cc = c[sel]
        a, b, e = ci[sel], cj[sel], ck[sel]
        if name == "top":      # 4 5 6 7
            q = (pid(a, b, e + 1), pid(a + 1, b, e + 1), pid(a + 1, b + 1, e + 1), pid(a, b + 1, e + 1))
        elif name == "bottom":  # 0 3 2 1
            q = (pid(a, b, e), pid(a, b + 1, e), pid(a + 1, b + 1, e), pid(a + 1, b, e))
        elif name == "left":    # 0 1 5 4
            q = (pid(a, b, e), pid(a + 1, b, e), pid(a + 1, b, e + 1), pid(a, b, e + 1))
        elif name == "right":   # 3 7 6 2
            q = (pid(a, b + 1, e), pid(a, b + 1, e + 1), pid(a + 1, b + 1, e + 1), pid(a + 1, b + 1, e))
        elif name == "back":    # 0 4 7 3
            q = (pid(a, b, e), pid(a, b, e + 1), pid(a, b + 1, e + 1), pid(a, b + 1, e))
        else:                   # front: 1 2 6 5
            q = (pid(a + 1, b, e), pid(a + 1, b + 1, e), pid(a + 1, b + 1, e + 1), pid(a + 1, b, e + 1))
        faces.append(np.stack(q, axis=1).astype(np.int32))
        owner.append(cc.astype(np.int32))
        patches.append((name, start, int(cc.size)))
        start += int(cc.size)
    fpts = np.concatenate(faces, axis=0)
    mesh = PolyMesh(
        points=pts,
        face_offsets=(np.arange(fpts.shape[0] + 1, dtype=np.int64) * 4).astype(np.int32),
        face_points=fpts.ravel(),
        owner=np.concatenate(owner),
        neighbour=nb.astype(np.int32),
        n_cells=nc,
        patches=patches,
        kind="hex-jitter" if jitter > 0 else "hex",
        h=h,
    )
    if metrics:
        compute_metrics(mesh)
    return mesh


def _orient_outward(pts, tets, faces_local):
    """Orient each tet face (3 local vertex ids) so its normal points away
    from the tet's fourth vertex."""
    nt = tets.shape[0]
    out = np.empty((nt, 4, 3), dtype=np.int64)
    for fi, (a, b, c) in enumerate(faces_local):
        d = ({0, 1, 2, 3} - {a, b, c}).pop()
        A, B, Cc, D = (pts[tets[:, x]] for x in (a, b, c, d))
        nrm = _cross(B - A, Cc - A)
        s = _dot(nrm, D - A)
        flip = s > 0
        tri = np.stack((tets[:, a], tets[:, b], tets[:, c]), axis=1)
        tri[flip] = tri[flip][:, [0, 2, 1]]
        out[:, fi, :] = tri
    return out


def tet_mesh(n: int, length: float = 1.0, metrics: bool = True) -> PolyMesh:
    """``n^3`` hexes, each split into 6 tetrahedra along its main diagonal
    (all cubes use the same diagonal, so the split is conforming).  Cells of
    cube ``q`` are ``6q .. 6q+5``; internal faces are ordered by owner then
    neighbour, boundary faces (one patch, ``walls``) by owner."""
    base = hex_mesh(n, length, metrics=False)
    pts = base.points
    n1 = n + 1
    nc_hex = n ** 3
    c = np.arange(nc_hex, dtype=np.int64)
    ci, cj, ck = c % n, (c // n) % n, c // (n * n)

    def corner(a, b, e):
        return (ci + a) + n1 * ((cj + b) + n1 * (ck + e))

    perms = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))
    tets = np.empty((nc_hex, 6, 4), dtype=np.int64)
    for t, p in enumerate(perms):
        v = [0, 0, 0]
        ids = [corner(0, 0, 0)]
        for ax in p:
            v[ax] = 1
            ids.append(corner(*v))
        tets[:, t, :] = np.stack(ids, axis=1)
    tets = tets.reshape(-1, 4)
    nt = tets.shape[0]
    fl = _orient_outward(pts, tets, ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)))
    allf = fl.reshape(-1, 3)
    cell_of = np.repeat(np.arange(nt, dtype=np.int64), 4)
    key = np.sort(allf, axis=1)
    order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    ks = key[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    first = np.ones(order.size, dtype=bool)
    first[1:] = ~same
    grp = np.cumsum(first) - 1
    ngrp = int(grp[-1]) + 1
    gsize = np.bincount(grp, minlength=ngrp)
    assert gsize.max() <= 2
    gstart = np.flatnonzero(first)
    inst0 = order[gstart]
    internal = gsize == 2
    inst1 = np.where(internal, order[np.minimum(gstart + 1, order.size - 1)], -1)
    c0 = cell_of[inst0]
    c1 = np.where(internal, cell_of[np.maximum(inst1, 0)], -1)
    # internal faces: owner = lower cell, oriented as the owner's instance
    ii = np.flatnonzero(internal)
    a0, a1 = c0[ii], c1[ii]
    own_i = np.minimum(a0, a1)
    nei_i = np.maximum(a0, a1)
    own_inst = np.where(a0 < a1, inst0[ii], inst1[ii])
    srt = np.lexsort((nei_i, own_i))
    own_i, nei_i, own_inst = own_i[srt], nei_i[srt], own_inst[srt]
    bi = np.flatnonzero(~internal)
    b_own = c0[bi]
    b_inst = inst0[bi]
    bsrt = np.lexsort((b_inst, b_own))
    b_own, b_inst = b_own[bsrt], b_inst[bsrt]
    fpts = np.concatenate((allf[own_inst], allf[b_inst]), axis=0).astype(np.int32)
    nf = fpts.shape[0]
    mesh = PolyMesh(
        points=pts,
        face_offsets=(np.arange(nf + 1, dtype=np.int64) * 3).astype(np.int32),
        face_points=fpts.ravel(),
        owner=np.concatenate((own_i, b_own)).astype(np.int32),
        neighbour=nei_i.astype(np.int32),
        n_cells=int(nt),
        patches=[("walls", int(own_i.size), int(b_own.size))],
        kind="tet",
        h=length / n,
    )
    if metrics:
        compute_metrics(mesh)
    return mesh


def make_mesh(kind: str, n: int, seed: int = 12345) -> PolyMesh:
    if kind == "hex":
        return hex_mesh(n)
    if kind == "refined":
        return refined_hex_mesh(n)
    if kind == "checker":
        return refined_hex_mesh(n, lo=(0.2, 0.2, 0.2), hi=(0.8, 0.8, 0.8), checker=True)
    if kind in ("hex-jitter", "jitter"):
        return hex_mesh(n, jitter=0.2, seed=seed)
    if kind == "tet":
        return tet_mesh(n)
    raise ValueError(f"unknown mesh kind {kind!r}")


# ---------------------------------------------------------------------------
# general polyhedral meshes: metrics for any face size and cell valence
# ---------------------------------------------------------------------------

def face_centres_areas_general(points: np.ndarray, face_offsets: np.ndarray, face_points: np.ndarray):
    """Face centres and area vectors of faces of any size (grouped by size,
    each group through ``face_centres_areas``: the same operation order)."""
    nf = face_offsets.size - 1
    sizes = np.diff(face_offsets)
    Cf = np.empty((nf, 3))
    Sf = np.empty((nf, 3))
    for n in np.unique(sizes):
        sel = np.flatnonzero(sizes == n)
        idx = face_offsets[sel][:, None] + np.arange(n)[None, :]
        c, s = face_centres_areas(points, face_points[idx])
        Cf[sel] = c
        Sf[sel] = s
    return Cf, Sf


def cell_centres_volumes_general(mesh: PolyMesh, Cf: np.ndarray, Sf: np.ndarray):
    """Cell centres and volumes for any cell valence: the pyramid sums of
    ``cell_centres_volumes`` per cell in cells() face order."""
    offs, cf = mesh.cell_faces()
    nc = mesh.n_cells
    cnt = np.diff(offs)
    own = mesh.owner
    C = np.empty((nc, 3))
    V = np.empty(nc)
    for k in np.unique(cnt):
        cells = np.flatnonzero(cnt == k)
        tb = cf[offs[cells][:, None] + np.arange(k)[None, :]].astype(np.int64)
        cEst = np.zeros((cells.size, 3))
        for j in range(k):
            cEst += Cf[tb[:, j]]
        cEst /= float(k)
        Cc = np.zeros((cells.size, 3))
        Vc = np.zeros(cells.size)
        for j in range(k):
            f = tb[:, j]
            is_own = own[f] == cells
            cfj = Cf[f]
            d = np.where(is_own[:, None], cfj - cEst, cEst - cfj)
            pyr3 = _dot(Sf[f], d)
            pc = 0.75 * cfj + 0.25 * cEst
            Cc += pyr3[:, None] * pc
            Vc += pyr3
        ok = np.abs(Vc) > VSMALL
        C[cells] = np.where(ok[:, None], Cc / np.where(ok, Vc, 1.0)[:, None], cEst)
        V[cells] = Vc * (1.0 / 3.0)
    return C, V


def compute_metrics_general(mesh: PolyMesh) -> PolyMesh:
    Cf, Sf = face_centres_areas_general(mesh.points, mesh.face_offsets.astype(np.int64), mesh.face_points)
    mesh.Cf, mesh.Sf = Cf, Sf
    mesh.magSf = _mag(Sf)
    mesh.C, mesh.V = cell_centres_volumes_general(mesh, Cf, Sf)
    return mesh


def refined_hex_mesh(n: int, lo=(0.25, 0.25, 0.25), hi=(0.75, 0.75, 0.75), checker: bool = False,
                     length: float = 1.0) -> PolyMesh:
    """``n^3`` hex block with the cells whose centres lie in the box
    [lo, hi] split 2 x 2 x 2 (one level of 2:1 refinement, as a refinement
    tool leaves it); with ``checker`` only every other cell of the box
    ((i + j + k) even) is split.  A coarse cell next to refined cells has
    that side split into four faces, and the points of its refined
    neighbours on its edges and sides are points of its faces (hanging
    nodes), so transition cells carry 7 to 24 faces and up to 26 points
    (24 and 26 inside a checker box), and faces up to 8 points.  Planar
    faces; internal faces in upper-triangular order, one boundary patch."""
    N = 2 * n  # fine lattice cells per direction
    c = np.arange(n ** 3)
    ci, cj, ck = c % n, (c // n) % n, c // (n * n)
    h = length / n
    ctr = np.stack(((ci + 0.5) * h, (cj + 0.5) * h, (ck + 0.5) * h), axis=1)
    refine = np.all((ctr >= np.asarray(lo)) & (ctr <= np.asarray(hi)), axis=1)
    if checker:
        refine &= (ci + cj + ck) % 2 == 0
    # cells as fine-lattice boxes (i0, j0, k0, size), in coarse order with
    # each refined cell replaced by its 8 children
    boxes = []
    for q in range(n ** 3):
        i0, j0, k0 = 2 * ci[q], 2 * cj[q], 2 * ck[q]
        if refine[q]:
            for dk in range(2):
                for dj in range(2):
                    for di in range(2):
                        boxes.append((i0 + di, j0 + dj, k0 + dk, 1))
        else:
            boxes.append((i0, j0, k0, 2))
    boxes = np.array(boxes, dtype=np.int64)
    nc = boxes.shape[0]
    # the cell covering each fine-lattice cell
    owner_of = np.empty((N, N, N), dtype=np.int64)
    for cell, (i0, j0, k0, s) in enumerate(boxes):
        owner_of[k0:k0 + s, j0:j0 + s, i0:i0 + s] = cell
    # active points: corners of all cells
    N1 = N + 1
    active = np.zeros((N1, N1, N1), dtype=bool)
    for (i0, j0, k0, s) in boxes:
        for dk in (0, s):
            for dj in (0, s):
                for di in (0, s):
                    active[k0 + dk, j0 + dj, i0 + di] = True
    pid = -np.ones((N1, N1, N1), dtype=np.int64)
    kk, jj, ii = np.nonzero(active)
    order = np.lexsort((ii, jj, kk))
    pid[kk[order], jj[order], ii[order]] = np.arange(order.size)
    pts = np.stack((ii[order], jj[order], kk[order]), axis=1).astype(np.float64) * (length / N)

    def loop(axis, x0, a0, a1, b0, b1, outward_positive):
        """Active lattice points on the boundary of the rectangle
        {axis = x0, u in [a0, a1], v in [b0, b1]} (u, v the next two axes
        cyclically), counter-clockwise about +axis, reversed for -axis."""
        u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
        path = []
        for u in range(a0, a1):
            path.append((u, b0))
        for v in range(b0, b1):
            path.append((a1, v))
        for u in range(a1, a0, -1):
            path.append((u, b1))
        for v in range(b1, b0, -1):
            path.append((a0, v))
        ids = []
        for u, v in path:
            p = [0, 0, 0]
            p[axis], p[u_ax], p[v_ax] = x0, u, v
            q = pid[p[2], p[1], p[0]]
            if q >= 0:
                ids.append(int(q))
        return ids if outward_positive else ids[::-1]

    internal = {}  # (owner, neighbour) -> list of faces (point lists)
    boundary = []  # (owner, points)
    for cell, (i0, j0, k0, s) in enumerate(boxes):
        lo3 = (i0, j0, k0)
        for axis in range(3):
            u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
            for side in (0, 1):
                x0 = lo3[axis] + (s if side else 0)
                # the fine-lattice cells across this side, per unit square
                groups = {}
                for a in range(lo3[u_ax], lo3[u_ax] + s):
                    for b in range(lo3[v_ax], lo3[v_ax] + s):
                        q = [0, 0, 0]
                        q[axis] = x0 if side else x0 - 1
                        q[u_ax], q[v_ax] = a, b
                        if q[axis] < 0 or q[axis] >= N:
                            other = -1
                        else:
                            other = int(owner_of[q[2], q[1], q[0]])
                        groups.setdefault(other, []).append((a, b))
                for other, sq in groups.items():
                    a0 = min(a for a, _ in sq)
                    a1 = max(a for a, _ in sq) + 1
                    b0 = min(b for _, b in sq)
                    b1 = max(b for _, b in sq) + 1
                    if other < 0:
                        boundary.append((cell, loop(axis, x0, a0, a1, b0, b1, side == 1)))
                    elif cell < other:  # the owner writes the face, normal out of it
                        internal.setdefault((cell, other), []).append(loop(axis, x0, a0, a1, b0, b1, side == 1))
    keys = sorted(internal)
    faces, owner, neigh = [], [], []
    for (o, nb) in keys:
        for f in internal[(o, nb)]:
            faces.append(f)
            owner.append(o)
            neigh.append(nb)
    nfi = len(faces)
    boundary.sort(key=lambda t: t[0])
    for o, f in boundary:
        faces.append(f)
        owner.append(o)
    offs = np.concatenate(([0], np.cumsum([len(f) for f in faces]))).astype(np.int32)
    mesh = PolyMesh(points=pts, face_offsets=offs, face_points=np.concatenate(faces).astype(np.int32),
                    owner=np.array(owner, np.int32), neighbour=np.array(neigh, np.int32), n_cells=nc,
                    patches=[("walls", nfi, len(faces) - nfi)], kind="hex-refined", h=h)
    return compute_metrics_general(mesh)
