"""Learned-normal form: what the trained network gains over the method
without it, and that the form keeps the volume exactly.

The network shipped in geometricvofext_gb300/data/normal_net.npz was trained
on the GPU by the package's own tensor-core forward / backward kernels
(``python -m geometricvofext_gb300.mlp``: 2^21 samples, 6 epochs, seed 1).
"""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from geometricvofext_gb300 import capi, harness as H, meshgen as mg, mlp  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

CTRL = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=False)


def _angles(n, ref):
    c = (n * ref).sum(1) / np.maximum(np.linalg.norm(n, axis=1), 1e-30)
    return np.degrees(np.arccos(np.clip(c, -1.0, 1.0)))


@pytest.mark.parametrize("sphere_percent", [0, 100])
def test_network_normals_beat_least_squares_on_hexes(sphere_percent):
    W, b = mlp.load_weights()
    mesh = mg.make_mesh("hex", 32)
    X, T = mlp.make_samples([mesh], 4096, seed=424242, sphere_percent=sphere_percent)
    nn, dc = mlp.predict_normals(W, b, X)
    Th = T.cpu().numpy()
    a_net = _angles(nn.cpu().numpy(), Th[:, :3])
    a_ls = _angles(X.float().cpu().numpy()[:, mlp.LS_SLOT:mlp.LS_SLOT + 3], Th[:, :3])
    # held-out planes / spheres: several times more accurate than least squares
    assert a_net.mean() < 0.5 * a_ls.mean(), (a_net.mean(), a_ls.mean())
    assert np.median(np.abs(dc.cpu().numpy() - Th[:, 3])) < 0.02


def _learned(mesh, **kw):
    g = capi.Simplic(mesh, precision=capi.PRECISION_LEARNED, **CTRL, **kw)
    W, b = mlp.load_weights()
    g.set_network(W, b)
    return g


def test_learned_form_matches_cell_volumes_and_uses_the_network():
    mesh = mg.make_mesh("hex", 24)
    a = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    g = _learned(mesh)
    g.reconstruct(a)
    cells, _ = g.mixed()
    # about half the cells take the network's normal (117 of 236 here); the
    # others are those where it fits the neighbours' volume fractions or the
    # face fluxes across the shared faces worse than least squares does
    used = g.network_stats()
    assert used >= 0.4 * len(cells), (used, len(cells))
    N, D, _, _ = g.interface()
    o = O.Oracle(mesh, **CTRL)
    worst = max(abs(o.calc_sub_cell(c, N[c], D[c])[1] - a[c]) for c in cells)
    assert worst <= 1e-11, worst


def test_learned_form_lowers_shape_error_at_equal_volume():
    """64^3 deformation over t in [0, 3]: the learned form's L1 shape error is
    below the plain FP64 form's, volume conserved to 1e-12 in both."""
    mesh = mg.make_mesh("hex", 64)
    alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    steps = int(math.ceil(3.0 / dt - 1e-9))
    dt = 3.0 / steps
    vol0 = float(np.sum(alpha0 * mesh.V))
    dev = torch.device("cuda", 0)
    phi0 = torch.from_numpy(flow.phi0).to(dev)
    U0 = torch.from_numpy(flow.U0).to(dev)
    Ub = torch.zeros((mesh.n_boundary_faces, 3), dtype=torch.float64, device=dev)
    phi, U = torch.empty_like(phi0), torch.empty_like(U0)
    res = {}
    for name in ("plain", "learned"):
        stream = torch.cuda.Stream(dev)
        torch.cuda.synchronize(dev)
        if name == "learned":
            g = _learned(mesh, stream=stream.cuda_stream)
        else:
            g = capi.Simplic(mesh, stream=stream.cuda_stream, **CTRL)
        g.set_alpha(alpha0)
        with torch.cuda.stream(stream):
            for k in range(steps):
                f = H.time_factor((k + 1) * dt, dt, flow.period)
                torch.mul(phi0, f, out=phi)
                torch.mul(U0, f, out=U)
                g.reconstruct_resident()
                g.advect_resident(phi, U, dt, U_boundary=Ub)
        g.synchronize()
        res[name] = H.errors(g.get_alpha(), alpha0, mesh.V, vol0)
    for e in res.values():
        assert abs(e.volume_error) <= 1e-12
    assert res["learned"].shape_error < res["plain"].shape_error, (res["learned"], res["plain"])


def _cell_points(mesh):
    """Points of every cell (the union of its faces' points)."""
    fo, fp = mesh.face_offsets, mesh.face_points
    pts = [set() for _ in range(mesh.n_cells)]
    for f in range(mesh.n_faces):
        ps = fp[fo[f]:fo[f + 1]]
        pts[mesh.owner[f]].update(ps.tolist())
        if f < mesh.n_internal_faces:
            pts[mesh.neighbour[f]].update(ps.tolist())
    return pts


@pytest.mark.parametrize("kind,n", [("hex", 12), ("jitter", 10), ("tet", 6)])
def test_step_network_inputs_follow_the_feature_definition(kind, n):
    """The rows the step feeds the network: the cell (alpha) and its 30
    nearest point neighbours by (distance rounded to h^2/1024, id), each as
    alpha_j - alpha_c and (C_j - C_c)/h in BF16, then the FP32 least-squares
    normal of those values.  The differences are taken in FP64 and rounded
    to FP32; the squared distance and the scaling by 1/h are FP32 products."""
    from oracle import mlp_oracle as MO

    mesh = mg.make_mesh(kind, n)
    a = H.sphere_alpha(mesh, (0.45, 0.5, 0.55), 0.27)
    W, b = mlp.load_weights()
    g = capi.Simplic(mesh, precision=capi.PRECISION_LEARNED, **CTRL)
    g.set_network(W, b)
    g.reconstruct(a)
    mixed, _ = g.mixed()
    cells, X = g.network_inputs()
    np.testing.assert_array_equal(cells, mixed)
    Xf = (X.astype(np.uint32) << 16).view(np.float32)
    cp = _cell_points(mesh)
    pc = {}
    for c, ps in enumerate(cp):
        for p in ps:
            pc.setdefault(p, []).append(c)
    C, V = mesh.C, mesh.V
    for row, c in enumerate(cells):
        st = sorted({x for p in cp[c] for x in pc[p]} - {c})
        hc = np.cbrt(V[c])
        ih2 = np.float32(1.0) / np.float32(hc * hc)
        ih = np.float32(1.0 / hc)
        keys = []
        for x in st:
            f = (C[x] - C[c]).astype(np.float32)
            q = (f[0] * f[0] + f[1] * f[1]) + f[2] * f[2]
            d2 = np.rint((q * ih2) * np.float32(1024.0))
            keys.append((float(d2), x))
        sel = [x for _, x in sorted(keys)[:30]]
        want = np.zeros(124, dtype=np.float32)
        want[0] = np.float32(a[c])
        t, v = [], []
        for k, x in enumerate(sel, start=1):
            rel = (C[x] - C[c]).astype(np.float32) * ih
            want[4 * k] = np.float32(a[x] - a[c])
            want[4 * k + 1:4 * k + 4] = rel
            t.append(rel)
            v.append(np.float32(a[x] - a[c]))
        np.testing.assert_array_equal(Xf[row, :124], MO.bf16(want), err_msg=f"cell {c}")
        # least-squares normal of a + g.t over the centre and the slots
        A = np.hstack([np.ones((len(t) + 1, 1)), np.vstack([np.zeros(3), np.array(t, dtype=np.float64)])])
        rhs = np.concatenate([[0.0], np.array(v, dtype=np.float64)])
        sol = np.linalg.lstsq(A, rhs, rcond=None)[0]
        grad = sol[1:]
        nrm = -grad / max(np.linalg.norm(grad), 1e-30)
        assert np.abs(Xf[row, 124:127] - nrm).max() < 2e-2, (c, Xf[row, 124:127], nrm)
        assert Xf[row, 127] == 0.0


def _cube_fraction(a, m):
    """Fraction of the unit cube below sum m_i u_i = a (m sorted, sum 1)."""
    if a <= 0.0:
        return 0.0
    if a >= 1.0:
        return 1.0
    flip = a > 0.5
    if flip:
        a = 1.0 - a
    # inclusion-exclusion over the cube corners
    tot = 0.0
    for i in range(2):
        for j in range(2):
            for k in range(2):
                t = a - (i * m[0] + j * m[1] + k * m[2])
                if t > 0:
                    tot += (-1) ** (i + j + k) * t ** 3
    F = tot / (6.0 * m[0] * m[1] * m[2])
    return 1.0 - F if flip else F


def _residual(n, X, A):
    """Local volume residual of normal n for one network row (the test the
    learned form applies): cubes of the cell's size on the cell and its
    neighbours, the plane through the cell's cube at its volume fraction."""
    p = np.abs(n) / np.abs(n).sum()
    p = np.maximum(p, 1e-4)
    p /= p.sum()
    m = np.sort(p)
    ps = np.copysign(p, n)
    ac = A[0]
    lo, hi = 0.0, 1.0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if _cube_fraction(mid, m) < ac:
            lo = mid
        else:
            hi = mid
    a0 = 0.5 * (lo + hi)
    R = 0.0
    for k in range(1, 31):
        r = X[4 * k + 1:4 * k + 4]
        if not r.any():
            continue
        R += abs(_cube_fraction(a0 - ps @ r, m) - (ac + A[k]))
    return R


def _cube_plane(n, alpha):
    """(signed coefficients p, plane constant a) of the cube [0,1]^3 cut at
    volume fraction alpha with normal n (the frame of the learned form)."""
    p = np.abs(n) / np.abs(n).sum()
    p = np.maximum(p, 1e-4)
    p /= p.sum()
    m = np.sort(p)
    lo, hi = 0.0, 1.0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if _cube_fraction(mid, m) < alpha:
            lo = mid
        else:
            hi = mid
    return np.copysign(p, n), 0.5 * (lo + hi)


def _square_fraction(b, q1, q2):
    lo, hi = min(q1, q2), max(q1, q2)
    s = lo + hi
    if b <= 0:
        return 0.0
    if b >= s:
        return 1.0
    if b < lo:
        return b * b / (2 * lo * hi)
    if b <= hi:
        return (b - 0.5 * lo) / hi
    return 1.0 - (s - b) ** 2 / (2 * lo * hi)


def _face_mismatch(n, X, A):
    """Face-flux mismatch of normal n for one network row: on each face with
    a face neighbour, the part of the face below the cell's plane against
    the part below the neighbour's own plane of the same normal."""
    ac = A[0]
    p, a0 = _cube_plane(n, ac)
    R = 0.0
    for k in range(1, 31):
        r = X[4 * k + 1:4 * k + 4]
        if not r.any():
            continue
        axis = int(np.argmax(np.abs(r)))
        rest = np.abs(r).sum() - abs(r[axis])
        if not (0.75 < abs(r[axis]) < 1.25 and rest < 0.25):
            continue
        sigma = 1.0 if r[axis] > 0 else -1.0
        _, aj0 = _cube_plane(n, ac + A[k])
        q = [abs(p[i]) for i in range(3) if i != axis]

        def part(a, sg):
            u = 1.0 if sg * p[axis] > 0 else 0.0
            return _square_fraction(a - abs(p[axis]) * u, q[0], q[1])

        R += abs(part(a0, sigma) - part(aj0, -sigma))
    return R


def test_network_normal_falls_back_when_it_raises_the_volume_residual():
    """A network forced to answer +x everywhere: only cells where that normal
    fits the neighbourhood's volume fractions and its face fluxes about as
    well as the least-squares normal take it (neither the local volume
    residual nor the face-flux mismatch more than gate_tol above the least-
    squares normal's); the others keep the least-squares normal."""
    mesh = mg.make_mesh("hex", 16)
    a = H.sphere_alpha(mesh, (0.5, 0.5, 0.5), 0.3)
    W = np.zeros((4, 128, 128), np.float32)
    b = np.zeros((4, 128), np.float32)
    b[3, 0] = 50.0  # y = (50, 0, 0, 0): normalise(n_ls + y[0:3]) is nearly +x
    g = capi.Simplic(mesh, precision=capi.PRECISION_LEARNED, **CTRL)
    g.set_network(W, b, gate_tol=capi.GATE_TOL)
    g.reconstruct(a)
    cells, X, Arows = g.network_inputs(alphas=True)
    Xf = (X.astype(np.uint32) << 16).view(np.float32)
    N, _, _, _ = g.interface()
    used = g.network_stats()
    gm = capi.Simplic(mesh, precision=capi.PRECISION_MIXED, **CTRL)
    gm.reconstruct(a)
    Nls, _, _, _ = gm.interface()
    took = np.zeros(len(cells), bool)
    nls = []
    for row, c in enumerate(cells):
        nl = Xf[row, 124:127].astype(np.float64) + np.array([50.0, 0.0, 0.0])
        nl /= np.linalg.norm(nl)
        nls.append(nl)
        took[row] = np.abs(N[c] - nl).max() < 1e-6
    assert took.sum() == used
    assert 0 < used < 0.5 * len(cells), (used, len(cells))
    checked = 0
    for row, c in enumerate(cells):
        x = Xf[row].astype(np.float64)
        A = Arows[row].astype(np.float64)
        assert A[0] == np.float32(a[c])
        nl = nls[row]
        rl, rs = _residual(nl, x, A), _residual(Nls[c], x, A)
        fl_, fs = _face_mismatch(nl, x, A), _face_mismatch(Nls[c], x, A)
        margin = rl - (rs + capi.GATE_TOL)
        fmargin = fl_ - (fs + capi.GATE_TOL)
        if abs(margin) < 1e-4 or abs(fmargin) < 1e-4:
            continue  # FP64 here, FP32 on the device
        checked += 1
        assert took[row] == (margin <= 0 and fmargin <= 0), (c, rl, rs, fl_, fs)
        if not took[row]:
            np.testing.assert_allclose(N[c], Nls[c], atol=1e-5)
    assert checked > 0.8 * len(cells)
