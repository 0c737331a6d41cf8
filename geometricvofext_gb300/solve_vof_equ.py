"""Host-side mirror of the reference ``solveVofEqu`` facade.

``SolveVofEqu`` has the reference object's construction and methods
(src/SimPLIC/solveVofEqu/solveVofEqu.H:118-211): it is built from the
volume fraction, face flux and velocity (held by reference and read at each
call), reads its controls from the ``solvers { "alpha.*" { ... } }`` entry of
an fvSolution dictionary (solveVofEqu.C:68 -> reconstruction.C:502-516,
advection.C:455-457), and forwards ``reconstruct()`` / ``advect(Sp, Su)`` to
the CUDA library.  Errors raise ``SimplicError`` instead of aborting.
"""

from __future__ import annotations

import re
from typing import Any, Dict, Optional, Union

import numpy as np

from . import capi


# ---------------------------------------------------------------------------
# a small OpenFOAM dictionary reader
# ---------------------------------------------------------------------------

def _tokens(text: str):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    return re.findall(r'"[^"]*"|[{};()]|[^\s{};()]+', text)


def _value(tok: str) -> Any:
    low = tok.lower()
    if low in ("true", "on", "yes"):
        return True
    if low in ("false", "off", "no", "none"):
        return False
    try:
        if re.fullmatch(r"[+-]?\d+", tok):
            return int(tok)
        return float(tok)
    except ValueError:
        return tok.strip('"')


def parse_dictionary(text: str) -> Dict[str, Any]:
    toks = _tokens(text)
    pos = 0

    def parse_block() -> Dict[str, Any]:
        nonlocal pos
        d: Dict[str, Any] = {}
        while pos < len(toks):
            t = toks[pos]
            if t == "}":
                pos += 1
                return d
            key = t
            pos += 1
            if pos < len(toks) and toks[pos] == "{":
                pos += 1
                d[key] = parse_block()
                continue
            vals = []
            depth = 0
            while pos < len(toks) and not (toks[pos] == ";" and depth == 0):
                if toks[pos] == "(":
                    depth += 1
                elif toks[pos] == ")":
                    depth -= 1
                vals.append(toks[pos])
                pos += 1
            pos += 1  # ';'
            d[key] = _value(vals[0]) if len(vals) == 1 else [_value(v) for v in vals]
        return d

    return parse_block()


def solver_dict(fv_solution: Union[str, Dict[str, Any]], field: str = "alpha.water") -> Dict[str, Any]:
    """``mesh.solverDict(field)``: the exact key, else the last regex key of
    ``solvers`` that matches the whole field name."""
    if isinstance(fv_solution, str):
        if "{" not in fv_solution:
            with open(fv_solution) as fh:
                fv_solution = fh.read()
        fv_solution = parse_dictionary(fv_solution)
    solvers = fv_solution.get("solvers", fv_solution)
    if field in solvers:
        return solvers[field]
    for key in reversed(list(solvers.keys())):
        if key.startswith('"') and re.fullmatch(key.strip('"'), field):
            return solvers[key]
    raise KeyError(f"no solver entry for {field}")


_ORIENT = {
    "alphaGrad": capi.ORIENTATION_ALPHA_GRAD,
    "isoAlphaGrad": capi.ORIENTATION_ISO_ALPHA_GRAD,
    "LS": capi.ORIENTATION_ISO_ALPHA_GRAD,
    "isoRDF": capi.ORIENTATION_ISO_RDF,
    "RDF": capi.ORIENTATION_ISO_RDF,
}


def controls_from_dict(d: Dict[str, Any]) -> capi.Controls:
    """The dictionary lookups of reconstruction.C:502-516 and
    advection.C:455-457 with the reference defaults; an unknown
    orientationMethod is an error (reconstruction.C:610-625)."""
    c = capi.default_controls()
    c.mixed_cell_tol = float(d.get("mixedCellTol", 1e-8))
    c.write_plic_fields = int(bool(d.get("writePlicFields", False)))
    c.split_warped_face = int(bool(d.get("splitWarpedFace", False)))
    om = str(d.get("orientationMethod", "isoAlphaGrad"))
    if om not in _ORIENT:
        raise ValueError(f"Orientation vector calculation method '{om}' is not valid")
    c.orientation_method = _ORIENT[om]
    c.map_alpha_field = int(bool(d.get("mapAlphaField", False)))
    c.iso_rdf_tol = float(d.get("tol", 1e-6))
    c.iso_rdf_rel_tol = float(d.get("relTol", 0.1))
    c.iso_rdf_iterations = int(d.get("iterations", 5))
    c.n_alpha_bounds = int(d.get("nAlphaBounds", 10))
    c.snap_tol = float(d.get("snapTol", 0.0))
    c.clip = int(bool(d.get("clip", True)))
    # the form of the step (no counterpart in the reference)
    prec = str(d.get("precision", "plain"))
    forms = {"plain": capi.PRECISION_PLAIN_FP64, "mixed": capi.PRECISION_MIXED, "learned": capi.PRECISION_LEARNED}
    if prec not in forms:
        raise ValueError(f"precision '{prec}' is not plain, mixed or learned")
    c.precision = forms[prec]
    return c


# ---------------------------------------------------------------------------
# the facade
# ---------------------------------------------------------------------------

class Reconstruction:
    """Read-only view of the reconstruction state (reconstruction.H:281-399)."""

    def __init__(self, s: "SolveVofEqu"):
        self._s = s

    def mixed_cells(self) -> np.ndarray:
        return self._s._h.mixed()[0]

    def cell_status(self) -> np.ndarray:
        return self._s._h.mixed()[1]

    def _iface(self):
        return self._s._h.interface()

    def interfaceN(self):
        return self._iface()[0]

    def interfaceD(self):
        return self._iface()[1]

    def interfaceC(self):
        return self._iface()[2]

    def interfaceS(self):
        return self._iface()[3]

    def face_flatness(self):
        return self._s._h.face_flatness()

    def is_a_mixed_cell(self, c: int) -> bool:
        a = self._s.alpha1[c]
        t = self._s._tol
        return t < a < 1.0 - t

    def reconstruction_time(self) -> float:
        return self._s._h.timers()[0]


class SolveVofEqu:
    """GPU drop-in for ``geometricVofExt::SimPLIC::solveVofEqu``.

    alpha1 is modified in place by ``advect``; phi, U (and the optional
    boundary values) are read at every call, so the caller updates those
    arrays in place between steps like OpenFOAM fields."""

    typeName = "solveVofEqu"

    def __init__(self, mesh, alpha1: np.ndarray, phi: np.ndarray, U: np.ndarray,
                 fv_solution: Union[str, Dict[str, Any]], field_name: str = "alpha.water",
                 U_boundary: Optional[np.ndarray] = None, alpha_boundary: Optional[np.ndarray] = None):
        self.mesh = mesh
        self.alpha1 = alpha1
        self.phi = phi
        self.U = U
        self.U_boundary = U_boundary
        self.alpha_boundary = alpha_boundary
        self._dict = solver_dict(fv_solution, field_name)
        ctrl = controls_from_dict(self._dict)
        self._tol = ctrl.mixed_cell_tol
        self._h = capi.Simplic(mesh, controls=ctrl)
        if ctrl.precision == capi.PRECISION_LEARNED:
            from . import mlp  # the shipped network; set_network() replaces it

            self._h.set_network(*mlp.load_weights())
        self.delta_t: Optional[float] = None
        self._old: Optional[np.ndarray] = None

    def set_network(self, W, b, gate_tol=capi.GATE_TOL) -> None:
        """The network of precision "learned" (no counterpart in the reference)."""
        self._h.set_network(W, b, gate_tol)

    # solveVofEqu.C:96-99
    def reconstruct(self) -> None:
        self._h.reconstruct(self.alpha1)

    # solveVofEquTemplates.C:35-43
    def advect(self, Sp: Optional[np.ndarray] = None, Su: Optional[np.ndarray] = None,
               alpha_old: Optional[np.ndarray] = None) -> None:
        if self.delta_t is None:
            raise RuntimeError("set delta_t (mesh.time().deltaT()) before advect")
        new = self._h.advect(self.alpha1, self.phi, self.U, self.delta_t, alpha_old=alpha_old,
                             U_boundary=self.U_boundary, alpha_boundary=self.alpha_boundary, Sp=Sp, Su=Su)
        self.alpha1[:] = new

    # solveVofEqu.C:102-105 -> reconstruction.C:725-784.  Without a plane
    # (a static mesh) there is nothing to map; after a refinement, on a
    # solver for the new mesh, the mapped interfaceN / interfaceD give the
    # new alpha of cells within [lower, upper] (dynamicMeshDict levels).
    def map_alpha_field(self, normal: Optional[np.ndarray] = None, distance: Optional[np.ndarray] = None,
                        lower: float = 0.001, upper: float = 0.999) -> None:
        if normal is None or not self._dict.get("mapAlphaField", False):
            return
        self.alpha1[:] = self._h.map_alpha_field(self.alpha1, normal, distance, lower, upper)

    # reconstruction::interface (reconstruction.C:787-835)
    def interface(self):
        """PLIC polygons of the last reconstruct: (offsets, points, cells)."""
        return self._h.interface_polygons()

    def alpha(self) -> np.ndarray:
        return self.alpha1

    def dict(self) -> Dict[str, Any]:
        return self._dict

    def get_rho_phi(self, rho1: float, rho2: float) -> np.ndarray:
        return self._h.rho_phi(rho1, rho2, self.phi)

    def alpha_phi(self) -> np.ndarray:
        return self._h.alpha_phi()

    def reconstructor(self) -> Reconstruction:
        return Reconstruction(self)

    def reconstruction_time(self) -> float:
        return self._h.timers()[0]

    def advection_time(self) -> float:
        return self._h.timers()[1]

    def alpha_mapping_time(self) -> float:
        return self._h.timers()[2]
