"""mapAlphaField (reconstruction.C:725-784) after a 2:1 refinement: every
child of an interface cell carries its parent's plane (the mesh mapper
copies interfaceN / interfaceD) and gets the volume fraction that plane
cuts from it.  A plane's cut volume is additive over a partition of the
parent, so the children's volumes add up to the parent's cut volume.

CPU: the oracle on a coarse 8^3 mesh and its 16^3 refinement.  GPU: the
CUDA entry point equals the oracle bit for bit (host and device arrays).
"""

import numpy as np
import pytest

from geometricvofext_gb300 import capi, harness as H, meshgen as mg
from oracle import oracle as O

LOWER, UPPER = 1e-8, 1.0 - 1e-8


def _refined_case(n=8):
    coarse = mg.make_mesh("hex", n)
    a = H.sphere_alpha(coarse, (0.45, 0.5, 0.55), 0.27)
    o = O.Oracle(coarse)
    o.reconstruct(a)
    N, D, _, _ = o.interface()
    cells, st = o.mixed()
    fine = mg.make_mesh("hex", 2 * n)
    c = np.arange(fine.n_cells)
    i, j, k = c % (2 * n), (c // (2 * n)) % (2 * n), c // (4 * n * n)
    parent = (i // 2) + n * ((j // 2) + n * (k // 2))
    return coarse, fine, parent, a, N, D, cells[st == 0]


def test_children_add_up_to_the_parent_cut():
    coarse, fine, parent, a, N, D, cut = _refined_case()
    of = O.Oracle(fine)
    a_map = of.map_alpha_field(a[parent], N[parent], D[parent], LOWER, UPPER)
    oc = O.Oracle(coarse)
    for c in cut:
        kids = np.flatnonzero(parent == c)
        st, vof, _, _ = oc.calc_sub_cell(c, N[c], D[c])
        vol_kids = float(np.sum(a_map[kids] * fine.V[kids]))
        assert abs(vol_kids - vof * coarse.V[c]) <= 1e-14, (c, vol_kids, vof * coarse.V[c])
    # cells outside [lower, upper] keep their mapped value
    keep = (a[parent] < LOWER) | (a[parent] > UPPER)
    np.testing.assert_array_equal(a_map[keep], a[parent][keep])


@pytest.mark.gpu
def test_gpu_map_alpha_equals_the_oracle():
    torch = pytest.importorskip("torch")
    coarse, fine, parent, a, N, D, cut = _refined_case()
    want = O.Oracle(fine).map_alpha_field(a[parent], N[parent], D[parent], LOWER, UPPER)
    g = capi.Simplic(fine, map_alpha_field=1)
    got = g.map_alpha_field(a[parent], N[parent], D[parent], LOWER, UPPER)
    np.testing.assert_array_equal(got, want)
    # device arrays, in place
    dev = torch.device("cuda", 0)
    ad = torch.from_numpy(a[parent].copy()).to(dev)
    nd = torch.from_numpy(np.ascontiguousarray(N[parent])).to(dev)
    dd = torch.from_numpy(D[parent].copy()).to(dev)
    torch.cuda.synchronize()
    import ctypes as C

    dp = C.POINTER(C.c_double)
    rc = capi.load().simplic_map_alpha_field(g._h, C.cast(C.c_void_p(ad.data_ptr()), dp),
                                             C.cast(C.c_void_p(nd.data_ptr()), dp),
                                             C.cast(C.c_void_p(dd.data_ptr()), dp), LOWER, UPPER, capi.MEM_DEVICE)
    assert rc == 0
    np.testing.assert_array_equal(ad.cpu().numpy(), want)
    assert g.timers()[2] > 0.0  # alphaMappingTime
