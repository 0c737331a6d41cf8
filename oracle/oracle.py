"""ctypes binding of the SimPLIC CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker (and the timed CPU baseline); the product path
never imports it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class OracleMesh(C.Structure):
    _fields_ = [
        ("n_points", C.c_int32), ("n_faces", C.c_int32),
        ("n_internal_faces", C.c_int32), ("n_cells", C.c_int32),
        ("points", _dp), ("face_offsets", _ip), ("face_points", _ip),
        ("owner", _ip), ("neighbour", _ip),
        ("cell_centres", _dp), ("cell_volumes", _dp),
        ("face_centres", _dp), ("face_areas", _dp), ("face_mag_areas", _dp),
    ]


class OracleControls(C.Structure):
    _fields_ = [
        ("mixed_cell_tol", C.c_double), ("n_alpha_bounds", C.c_int32),
        ("snap_tol", C.c_double), ("clip", C.c_int32), ("n_threads", C.c_int32),
        ("orientation", C.c_int32), ("rdf_tol", C.c_double), ("rdf_rel_tol", C.c_double),
        ("rdf_iterations", C.c_int32), ("split_warped_face", C.c_int32),
    ]


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(
            os.path.getmtime(os.path.join(_HERE, f))
            for f in ("simplic_oracle.cpp", "simplic_oracle.h"))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(OracleMesh), C.POINTER(OracleControls)]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_reconstruct.argtypes = [C.c_void_p, _dp]
        L.oracle_advect.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp]
        L.oracle_n_mixed.restype = C.c_int32
        L.oracle_n_mixed.argtypes = [C.c_void_p]
        L.oracle_get_mixed.argtypes = [C.c_void_p, _ip, _ip]
        L.oracle_get_interface.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.oracle_get_alpha_phi.argtypes = [C.c_void_p, _dp]
        L.oracle_get_dvf.argtypes = [C.c_void_p, _dp]
        L.oracle_get_face_flatness.argtypes = [C.c_void_p, _dp]
        L.oracle_get_cut_faces.argtypes = [C.c_void_p, _u8p]
        L.oracle_get_stats.argtypes = [C.c_void_p, _dp, _ip]
        L.oracle_interface_polygons.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _ip]
        L.oracle_map_alpha_field.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double, C.c_double]
        L.oracle_plane_angle.restype = C.c_double
        L.oracle_plane_angle.argtypes = [C.c_double, C.c_double]
        L.oracle_rdf_iterations.restype = C.c_int32
        L.oracle_rdf_iterations.argtypes = [C.c_void_p]
        L.oracle_calc_sub_face.argtypes = [_dp, C.c_int32, _dp, C.c_double, _dp, _dp]
        L.oracle_calc_sub_cell.argtypes = [C.c_void_p, C.c_int32, _dp, C.c_double, _dp, _dp, _dp]
        L.oracle_find_signed_distance.argtypes = [C.c_void_p, C.c_int32, C.c_double, _dp, _dp, _dp, _dp]
        L.oracle_time_integrated_face_flux.restype = C.c_double
        L.oracle_time_integrated_face_flux.argtypes = [C.c_void_p, C.c_int32, _dp, C.c_double, C.c_double,
                                                       C.c_double, C.c_double, C.c_double]
        L.oracle_interpolate_U.argtypes = [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """The reference solveVofEqu object restated on the CPU (FP64)."""

    def __init__(self, mesh, mixed_cell_tol=1e-8, n_alpha_bounds=10, snap_tol=0.0,
                 clip=True, n_threads=1, orientation="isoAlphaGrad", rdf_tol=1e-6, rdf_rel_tol=0.1,
                 rdf_iterations=5, split_warped_face=False):
        L = lib()
        self.mesh = mesh
        self._keep = [
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
        k = self._keep
        self._m = OracleMesh(mesh.n_points, mesh.n_faces, mesh.n_internal_faces, mesh.n_cells,
                             _d(k[0]), _i(k[1]), _i(k[2]), _i(k[3]), _i(k[4]),
                             _d(k[5]), _d(k[6]), _d(k[7]), _d(k[8]), _d(k[9]))
        if orientation not in ("isoAlphaGrad", "isoRDF"):
            raise ValueError(f"orientation {orientation!r}")
        self._c = OracleControls(float(mixed_cell_tol), int(n_alpha_bounds), float(snap_tol),
                                 int(bool(clip)), int(n_threads), int(orientation == "isoRDF"),
                                 float(rdf_tol), float(rdf_rel_tol), int(rdf_iterations),
                                 int(bool(split_warped_face)))
        self._h = L.oracle_create(C.byref(self._m), C.byref(self._c))
        self.nc = mesh.n_cells
        self.nf = mesh.n_faces

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_destroy(h)
            self._h = None

    def reconstruct(self, alpha):
        a = _f64(alpha)
        lib().oracle_reconstruct(self._h, _d(a))

    def advect(self, alpha, phi, U, dt, alpha_old=None, U_boundary=None, alpha_boundary=None,
               Sp=None, Su=None):
        """Returns the new alpha (the input array is not modified)."""
        a = np.array(alpha, dtype=np.float64, copy=True)
        args = [_f64(x) for x in (alpha_old, phi, U, U_boundary, alpha_boundary, Sp, Su)]
        lib().oracle_advect(self._h, _d(a), _d(args[0]), _d(args[1]), _d(args[2]), _d(args[3]),
                            _d(args[4]), float(dt), _d(args[5]), _d(args[6]))
        return a

    def mixed(self):
        n = lib().oracle_n_mixed(self._h)
        cells = np.empty(n, np.int32)
        st = np.empty(n, np.int32)
        lib().oracle_get_mixed(self._h, _i(cells), _i(st))
        return cells, st

    def interface(self):
        n = np.empty((self.nc, 3)); d = np.empty(self.nc)
        c = np.empty((self.nc, 3)); s = np.empty((self.nc, 3))
        lib().oracle_get_interface(self._h, _d(n), _d(d), _d(c), _d(s))
        return n, d, c, s

    def alpha_phi(self):
        out = np.empty(self.nf)
        lib().oracle_get_alpha_phi(self._h, _d(out))
        return out

    def dvf(self):
        out = np.empty(self.nf)
        lib().oracle_get_dvf(self._h, _d(out))
        return out

    def face_flatness(self):
        out = np.empty(self.nf)
        lib().oracle_get_face_flatness(self._h, _d(out))
        return out

    def cut_faces(self):
        out = np.empty(self.nf, np.uint8)
        lib().oracle_get_cut_faces(self._h, out.ctypes.data_as(_u8p))
        return out

    def stats(self):
        t = np.empty(2)
        n = np.empty(2, np.int32)
        lib().oracle_get_stats(self._h, _d(t), _i(n))
        return float(t[0]), float(t[1]), int(n[0]), int(n[1])

    def map_alpha_field(self, alpha, normal, distance, lower, upper):
        """New alpha: cells with lower <= alpha <= upper get the volume
        fraction of their plane (normal, distance)."""
        a = np.array(alpha, dtype=np.float64, copy=True)
        lib().oracle_map_alpha_field(self._h, _d(a), _d(_f64(normal)), _d(_f64(distance)), float(lower),
                                     float(upper))
        return a

    def interface_polygons(self):
        """(offsets [n+1], points [np, 3], cells [n]) of the PLIC surface of
        the last reconstruct, ascending in cell"""
        nq, npt = C.c_int32(), C.c_int32()
        lib().oracle_interface_polygons(self._h, C.byref(nq), C.byref(npt), None, None, None)
        off = np.empty(nq.value + 1, np.int32)
        pts = np.empty((npt.value, 3))
        cells = np.empty(nq.value, np.int32)
        lib().oracle_interface_polygons(self._h, C.byref(nq), C.byref(npt), _i(off), _d(pts), _i(cells))
        return off, pts, cells

    def rdf_iterations(self):
        return int(lib().oracle_rdf_iterations(self._h))

    # unit-level
    def calc_sub_cell(self, cell, normal, distance):
        nrm = _f64(normal); vof = np.empty(1); c = np.empty(3); s = np.empty(3)
        st = lib().oracle_calc_sub_cell(self._h, int(cell), _d(nrm), float(distance), _d(vof), _d(c), _d(s))
        return st, float(vof[0]), c, s

    def find_signed_distance(self, cell, alpha, normal):
        nrm = _f64(normal); d = np.zeros(1); c = np.zeros(3); s = np.zeros(3)
        st = lib().oracle_find_signed_distance(self._h, int(cell), float(alpha), _d(nrm), _d(d), _d(c), _d(s))
        return st, float(d[0]), c, s

    def time_integrated_face_flux(self, face, normal, d, Un0, dt, phi, magSf):
        nrm = _f64(normal)
        return lib().oracle_time_integrated_face_flux(self._h, int(face), _d(nrm), float(d), float(Un0),
                                                      float(dt), float(phi), float(magSf))

    def interpolate_U(self, cell, x, U, U_boundary=None):
        out = np.empty(3)
        xx = _f64(x); UU = _f64(U); Ub = _f64(U_boundary)
        lib().oracle_interpolate_U(self._h, int(cell), _d(xx), _d(UU), _d(Ub), _d(out))
        return out


def calc_sub_face(points, normal, distance):
    p = _f64(points); nrm = _f64(normal); c = np.empty(3); a = np.empty(3)
    st = lib().oracle_calc_sub_face(_d(p), int(p.shape[0]), _d(nrm), float(distance), _d(c), _d(a))
    return st, c, a


def plane_angle(y, x):
    """The angle that orders the PLIC polygon points (an atan2 of correctly
    rounded operations only)."""
    return float(lib().oracle_plane_angle(float(y), float(x)))
