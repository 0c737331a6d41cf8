"""ctypes binding of ``libsimplic_cuda.so`` (the C ABI in include/simplic.h).

There is no CPU path behind this module: if the CUDA library cannot be built
or loaded, or no GPU is present, the calls raise.
"""

from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)

OK = 0
PRECISION_PLAIN_FP64 = 0
PRECISION_MIXED = 1
PRECISION_LEARNED = 2
# learned form: the network's normal is kept unless it raises the local
# volume residual (sum over the cell's 30 nearest neighbours) by more than this
GATE_TOL = 0.01
ORIENTATION_ALPHA_GRAD = 0
ORIENTATION_ISO_ALPHA_GRAD = 1
ORIENTATION_ISO_RDF = 2
MEM_HOST = 0
MEM_DEVICE = 1
ALPHA_UNCHANGED = 1


class SimplicError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"simplic error {code}: {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [
        ("n_points", C.c_int32), ("n_faces", C.c_int32),
        ("n_internal_faces", C.c_int32), ("n_cells", C.c_int32),
        ("points", _dp), ("face_offsets", _ip), ("face_points", _ip),
        ("owner", _ip), ("neighbour", _ip),
        ("cell_centres", _dp), ("cell_volumes", _dp),
        ("face_centres", _dp), ("face_areas", _dp), ("face_mag_areas", _dp),
    ]


class Controls(C.Structure):
    _fields_ = [
        ("mixed_cell_tol", C.c_double), ("orientation_method", C.c_int32),
        ("split_warped_face", C.c_int32), ("n_alpha_bounds", C.c_int32),
        ("snap_tol", C.c_double), ("clip", C.c_int32),
        ("write_plic_fields", C.c_int32), ("map_alpha_field", C.c_int32),
        ("precision", C.c_int32), ("record_cut_faces", C.c_int32),
        ("iso_rdf_tol", C.c_double), ("iso_rdf_rel_tol", C.c_double), ("iso_rdf_iterations", C.c_int32),
    ]


class StepInputs(C.Structure):
    _fields_ = [
        ("phi", _dp), ("U", _dp), ("U_boundary", _dp), ("alpha_boundary", _dp),
        ("Sp", _dp), ("Su", _dp), ("dt", C.c_double), ("flags", C.c_uint32),
    ]


_lib = None

EXPORTS = (
    "simplic_default_controls", "simplic_create", "simplic_destroy", "simplic_last_error",
    "simplic_reconstruct", "simplic_advect", "simplic_set_alpha", "simplic_reconstruct_resident",
    "simplic_advect_resident", "simplic_alpha_device", "simplic_get_alpha", "simplic_synchronize",
    "simplic_get_mixed_cells", "simplic_get_interface", "simplic_get_alpha_phi", "simplic_get_rho_phi",
    "simplic_get_face_flatness", "simplic_get_cut_faces", "simplic_timers", "simplic_stats",
    "simplic_set_kernel_timing", "simplic_kernel_times", "simplic_reset_kernel_times",
    "simplic_bound_info", "simplic_bound_profile", "simplic_mesh_info", "simplic_rdf_iterations", "simplic_get_interface_polygons",
    "simplic_map_alpha_field", "simplic_mixed_cells_noalloc", "simplic_mlp_gemm", "simplic_mlp_forward",
    "simplic_mlp_samples",
    "simplic_set_network", "simplic_network_stats", "simplic_network_info", "simplic_network_inputs",
)
N_KERNELS = 14


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_needed: bool = True):
    """Load (and if needed build) the CUDA library; raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB_PATH):
        raise ImportError(f"{_build.LIB_PATH} is missing; run geometricvofext_gb300.build.build()")
    L = C.CDLL(_build.LIB_PATH)
    h = C.c_void_p
    L.simplic_default_controls.argtypes = [C.POINTER(Controls)]
    L.simplic_default_controls.restype = None
    L.simplic_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(Controls), C.c_void_p, C.POINTER(C.c_void_p)]
    L.simplic_destroy.argtypes = [h]
    L.simplic_last_error.argtypes = [h]
    L.simplic_last_error.restype = C.c_char_p
    L.simplic_reconstruct.argtypes = [h, _dp]
    L.simplic_advect.argtypes = [h, _dp, _dp, C.POINTER(StepInputs)]
    L.simplic_set_alpha.argtypes = [h, C.c_void_p, C.c_int32]
    L.simplic_reconstruct_resident.argtypes = [h]
    L.simplic_advect_resident.argtypes = [h, C.POINTER(StepInputs)]
    L.simplic_alpha_device.argtypes = [h]
    L.simplic_alpha_device.restype = C.c_void_p
    L.simplic_get_alpha.argtypes = [h, C.c_void_p, C.c_int32]
    L.simplic_synchronize.argtypes = [h]
    L.simplic_get_mixed_cells.argtypes = [h, _ip, _ip, _ip]
    L.simplic_get_interface.argtypes = [h, _dp, _dp, _dp, _dp]
    L.simplic_get_alpha_phi.argtypes = [h, C.c_void_p, C.c_int32]
    L.simplic_get_rho_phi.argtypes = [h, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_int32]
    L.simplic_get_face_flatness.argtypes = [h, _dp]
    L.simplic_get_cut_faces.argtypes = [h, _u8p]
    L.simplic_timers.argtypes = [h, _dp, _dp, _dp]
    L.simplic_stats.argtypes = [h, _ip, _ip, _ip]
    L.simplic_set_kernel_timing.argtypes = [h, C.c_int32]
    L.simplic_kernel_times.argtypes = [h, _dp, C.POINTER(C.c_int64), C.POINTER(C.c_char_p)]
    L.simplic_reset_kernel_times.argtypes = [h]
    L.simplic_bound_info.argtypes = [h, _ip]
    L.simplic_bound_profile.argtypes = [h, _ip]
    L.simplic_mesh_info.argtypes = [h, _ip]
    L.simplic_rdf_iterations.argtypes = [h, _ip]
    L.simplic_get_interface_polygons.argtypes = [h, _ip, _ip, _ip, _dp, _ip]
    L.simplic_map_alpha_field.argtypes = [h, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int32]
    vp, i32 = C.c_void_p, C.c_int32
    L.simplic_mlp_gemm.argtypes = [vp, i32, vp, i32, i32, i32, i32, i32, vp, i32, vp, vp, i32, vp, i32, vp, i32,
                                   i32, vp, vp]
    L.simplic_mlp_forward.argtypes = [vp, vp, i32, vp, vp, vp, i32, vp, vp]
    L.simplic_mlp_samples.argtypes = [h, C.c_uint64, i32, i32, vp, vp]
    L.simplic_set_network.argtypes = [h, vp, vp, C.c_float]
    L.simplic_network_stats.argtypes = [h, _ip]
    L.simplic_network_info.argtypes = [h, _ip]
    L.simplic_network_inputs.argtypes = [h, C.c_int32, _ip, _ip, C.c_void_p, C.c_void_p]
    for name in EXPORTS:
        getattr(L, name)
    _lib = L
    return L


def default_controls() -> Controls:
    c = Controls()
    load().simplic_default_controls(C.byref(c))
    return c


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    """Host numpy array or a torch CUDA tensor -> raw pointer."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.cast(C.c_void_p(a.data_ptr()), _dp)
    return a.ctypes.data_as(_dp)


class Simplic:
    """One handle of the CUDA SimPLIC step (one reference solveVofEqu)."""

    def __init__(self, mesh, controls: Optional[Controls] = None, stream: Optional[int] = None, **overrides):
        L = load()
        ctrl = controls or default_controls()
        for k, v in overrides.items():
            if not hasattr(ctrl, k):
                raise TypeError(f"unknown control {k}")
            setattr(ctrl, k, v)
        self.controls = ctrl
        self.mesh = mesh
        keep = [
            np.ascontiguousarray(mesh.points, dtype=np.float64),
            np.ascontiguousarray(mesh.face_offsets, dtype=np.int32),
            np.ascontiguousarray(mesh.face_points, dtype=np.int32),
            np.ascontiguousarray(mesh.owner, dtype=np.int32),
            np.ascontiguousarray(mesh.neighbour, dtype=np.int32),
            np.ascontiguousarray(mesh.C, dtype=np.float64),
            np.ascontiguousarray(mesh.V, dtype=np.float64),
            np.ascontiguousarray(mesh.Cf, dtype=np.float64),
            np.ascontiguousarray(mesh.Sf, dtype=np.float64),
            np.ascontiguousarray(mesh.magSf, dtype=np.float64),
        ]
        ip = lambda a: a.ctypes.data_as(_ip)
        desc = MeshDesc(mesh.n_points, mesh.n_faces, mesh.n_internal_faces, mesh.n_cells,
                        _d(keep[0]), ip(keep[1]), ip(keep[2]), ip(keep[3]), ip(keep[4]),
                        _d(keep[5]), _d(keep[6]), _d(keep[7]), _d(keep[8]), _d(keep[9]))
        h = C.c_void_p()
        r = L.simplic_create(C.byref(desc), C.byref(ctrl), C.c_void_p(stream) if stream else None, C.byref(h))
        if r != OK:
            raise SimplicError(r, L.simplic_last_error(None).decode())
        self._h = h
        self.nc = mesh.n_cells
        self.nf = mesh.n_faces
        self.nfb = mesh.n_faces - mesh.n_internal_faces

    def close(self):
        if getattr(self, "_h", None):
            load().simplic_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, r):
        if r != OK:
            raise SimplicError(r, load().simplic_last_error(self._h).decode())

    # ----- drop-in (host arrays) -----
    def reconstruct(self, alpha):
        a = _f64(alpha)
        self._check(load().simplic_reconstruct(self._h, _d(a)))

    def advect(self, alpha, phi, U, dt, alpha_old=None, U_boundary=None, alpha_boundary=None,
               Sp=None, Su=None, unchanged=False):
        """Returns the new alpha (a copy; the input array is not modified)."""
        a = np.array(alpha, dtype=np.float64, copy=True)
        arrs = [_f64(x) for x in (alpha_old, phi, U, U_boundary, alpha_boundary, Sp, Su)]
        si = StepInputs(_d(arrs[1]), _d(arrs[2]), _d(arrs[3]), _d(arrs[4]), _d(arrs[5]), _d(arrs[6]),
                        float(dt), ALPHA_UNCHANGED if unchanged else 0)
        self._check(load().simplic_advect(self._h, _d(a), _d(arrs[0]), C.byref(si)))
        return a

    def advect_inplace(self, alpha: np.ndarray, phi, U, dt, U_boundary=None, unchanged=True):
        """Host API with caller-owned (ideally pinned) buffers; alpha is
        updated in place."""
        si = StepInputs(_ptr(phi), _ptr(U), _ptr(U_boundary), None, None, None, float(dt),
                        ALPHA_UNCHANGED if unchanged else 0)
        self._check(load().simplic_advect(self._h, _ptr(alpha), None, C.byref(si)))

    def reconstruct_ptr(self, alpha: np.ndarray):
        self._check(load().simplic_reconstruct(self._h, _ptr(alpha)))

    # ----- device-resident -----
    def set_alpha(self, alpha, device=False):
        if device:
            self._check(load().simplic_set_alpha(self._h, C.c_void_p(alpha.data_ptr()), MEM_DEVICE))
        else:
            a = _f64(alpha)
            self._check(load().simplic_set_alpha(self._h, a.ctypes.data_as(C.c_void_p), MEM_HOST))
            load().simplic_synchronize(self._h)

    def reconstruct_resident(self):
        self._check(load().simplic_reconstruct_resident(self._h))

    def advect_resident(self, phi, U, dt, U_boundary=None, alpha_boundary=None, Sp=None, Su=None):
        """phi / U / ... are torch CUDA tensors (device pointers)."""
        si = StepInputs(_ptr(phi), _ptr(U), _ptr(U_boundary), _ptr(alpha_boundary), _ptr(Sp), _ptr(Su),
                        float(dt), 0)
        self._check(load().simplic_advect_resident(self._h, C.byref(si)))

    def alpha_device_ptr(self) -> int:
        return load().simplic_alpha_device(self._h)

    def get_alpha(self) -> np.ndarray:
        out = np.empty(self.nc)
        self._check(load().simplic_get_alpha(self._h, out.ctypes.data_as(C.c_void_p), MEM_HOST))
        return out

    def synchronize(self):
        self._check(load().simplic_synchronize(self._h))

    # ----- accessors -----
    def mixed(self):
        n = C.c_int32()
        self._check(load().simplic_get_mixed_cells(self._h, C.byref(n), None, None))
        cells = np.empty(n.value, np.int32)
        st = np.empty(n.value, np.int32)
        self._check(load().simplic_get_mixed_cells(self._h, C.byref(n), cells.ctypes.data_as(_ip),
                                                   st.ctypes.data_as(_ip)))
        return cells, st

    def interface(self):
        n = np.empty((self.nc, 3)); d = np.empty(self.nc)
        c = np.empty((self.nc, 3)); s = np.empty((self.nc, 3))
        self._check(load().simplic_get_interface(self._h, _d(n), _d(d), _d(c), _d(s)))
        return n, d, c, s

    def alpha_phi(self) -> np.ndarray:
        out = np.empty(self.nf)
        self._check(load().simplic_get_alpha_phi(self._h, out.ctypes.data_as(C.c_void_p), MEM_HOST))
        return out

    def rho_phi(self, rho1: float, rho2: float, phi) -> np.ndarray:
        p = _f64(phi)
        out = np.empty(self.nf)
        self._check(load().simplic_get_rho_phi(self._h, float(rho1), float(rho2), p.ctypes.data_as(C.c_void_p),
                                               out.ctypes.data_as(C.c_void_p), MEM_HOST))
        return out

    def face_flatness(self) -> np.ndarray:
        out = np.empty(self.nf)
        self._check(load().simplic_get_face_flatness(self._h, _d(out)))
        return out

    def cut_faces(self) -> np.ndarray:
        out = np.empty(self.nf, np.uint8)
        self._check(load().simplic_get_cut_faces(self._h, out.ctypes.data_as(_u8p)))
        return out

    def timers(self):
        r, a, m = C.c_double(), C.c_double(), C.c_double()
        self._check(load().simplic_timers(self._h, C.byref(r), C.byref(a), C.byref(m)))
        return r.value, a.value, m.value

    def set_kernel_timing(self, enable: bool):
        self._check(load().simplic_set_kernel_timing(self._h, int(bool(enable))))

    def kernel_times(self):
        """{kernel name: (total ms of timed launches, launches)}"""
        ms = np.zeros(N_KERNELS)
        n = (C.c_int64 * N_KERNELS)()
        names = (C.c_char_p * N_KERNELS)()
        self._check(load().simplic_kernel_times(self._h, _d(ms), n, names))
        return {names[i].decode(): (float(ms[i]), int(n[i])) for i in range(N_KERNELS)}

    def reset_kernel_times(self):
        self._check(load().simplic_reset_kernel_times(self._h))

    def bound_info(self):
        """(passes, most overshooting cells in a pass, most dependency chains
        started from the ready queue in a pass, overflowed list code) of the
        last advect"""
        info = np.zeros(4, np.int32)
        self._check(load().simplic_bound_info(self._h, info.ctypes.data_as(_ip)))
        return tuple(int(x) for x in info)

    def bound_profile(self):
        """(most cells one warp ran in a row along a dependency chain, cells
        run in all passes, microseconds in the dependency phases, microseconds
        of the bounding launch) of the last advect"""
        info = np.zeros(4, np.int32)
        self._check(load().simplic_bound_profile(self._h, info.ctypes.data_as(_ip)))
        return tuple(int(x) for x in info)

    def mesh_info(self):
        """(common face count, lattice nx, ny, nz, box cells) found at create"""
        info = np.zeros(5, np.int32)
        self._check(load().simplic_mesh_info(self._h, info.ctypes.data_as(_ip)))
        return tuple(int(x) for x in info)

    # ----- learned-normal network -----
    def samples(self, seed, X, T, sphere_percent=50):
        """Training samples on this mesh into torch CUDA tensors X (bf16
        [n, 128]) and T (float32 [n, 4]); enqueued on the handle's stream."""
        self._check(load().simplic_mlp_samples(self._h, int(seed), X.shape[0], int(sphere_percent),
                                               C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr())))

    def set_network(self, W, b, gate_tol=GATE_TOL):
        """W [4, 128, 128] and b [4, 128] (float32, host) of the learned
        precision; a cell keeps its least-squares normal when the network's
        normal raises the local volume residual by more than gate_tol."""
        Wc = np.ascontiguousarray(W, dtype=np.float32)
        bc = np.ascontiguousarray(b, dtype=np.float32)
        self._check(load().simplic_set_network(self._h, Wc.ctypes.data_as(C.c_void_p), bc.ctypes.data_as(C.c_void_p),
                                               float(gate_tol)))

    def network_inputs(self, max_rows=None, alphas=False):
        """The network inputs of the last reconstruct, ascending in cell:
        (cells int32 [rows], X uint16 [rows, 128] BF16 bit patterns), and
        with alphas=True also the FP32 alpha rows of the fallback test
        (float32 [rows, 32])."""
        cap = self.nc if max_rows is None else int(max_rows)
        X = np.empty((max(cap, 1), 128), dtype=np.uint16)
        A = np.empty((max(cap, 1), 32), dtype=np.float32) if alphas else None
        cells = np.empty(max(cap, 1), dtype=np.int32)
        n = C.c_int32()
        self._check(load().simplic_network_inputs(self._h, cap, C.byref(n), cells.ctypes.data_as(_ip),
                                                  X.ctypes.data_as(C.c_void_p),
                                                  A.ctypes.data_as(C.c_void_p) if alphas else None))
        if alphas:
            return cells[: n.value], X[: n.value], A[: n.value]
        return cells[: n.value], X[: n.value]

    def network_stats(self):
        n = C.c_int32()
        self._check(load().simplic_network_stats(self._h, C.byref(n)))
        return n.value

    def network_info(self):
        """(cells that took the network's normal, network row capacity, mixed
        cells beyond the capacity that kept the least-squares normal) of the
        last reconstruct"""
        info = np.zeros(3, np.int32)
        self._check(load().simplic_network_info(self._h, info.ctypes.data_as(_ip)))
        return tuple(int(x) for x in info)

    def network_overflow(self):
        return self.network_info()[2]

    def map_alpha_field(self, alpha, normal, distance, lower, upper):
        """mapAlphaField on this (refined) mesh: a new alpha where cells with
        lower <= alpha <= upper take the volume fraction of their plane."""
        a = np.array(alpha, dtype=np.float64, copy=True)
        n, d = _f64(normal), _f64(distance)
        self._check(load().simplic_map_alpha_field(self._h, _d(a), _d(n), _d(d), float(lower), float(upper),
                                                   MEM_HOST))
        return a

    def interface_polygons(self):
        """The PLIC surface of the last reconstruct: (offsets [n+1],
        points [np, 3], cells [n]), one polygon per cut mixed cell,
        ascending in cell"""
        nq, npt = C.c_int32(), C.c_int32()
        self._check(load().simplic_get_interface_polygons(self._h, C.byref(nq), C.byref(npt), None, None, None))
        off = np.empty(nq.value + 1, np.int32)
        pts = np.empty((max(npt.value, 1), 3))
        cells = np.empty(max(nq.value, 1), np.int32)
        self._check(load().simplic_get_interface_polygons(self._h, C.byref(nq), C.byref(npt), off.ctypes.data_as(_ip),
                                                          _d(pts), cells.ctypes.data_as(_ip)))
        return off, pts[: npt.value], cells[: nq.value]

    def rdf_iterations(self):
        """isoRDF iterations of the last reconstruct (0 for least squares)"""
        n = C.c_int32()
        self._check(load().simplic_rdf_iterations(self._h, C.byref(n)))
        return n.value

    def stats(self):
        n, p, b = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(load().simplic_stats(self._h, C.byref(n), C.byref(p), C.byref(b)))
        return n.value, p.value, b.value
