"""PLIC surface output: the interface polygons of a reconstruct as a VTK
PolyData file (.vtp), the format the reference's ``plicSurface`` sampler
writes (``sampledPlicSurface``, ``tutorials/test/plicVofAdvectionFoam/
system/controlDict:44-68``: surfaceFormat vtp, fields alpha, U, cellIds).

The polygons come from ``Simplic.interface_polygons()`` (the C ABI's
``simplic_get_interface_polygons``): offsets, points and the cell of each
polygon.  Cell fields are sampled per polygon from its cell (the
sampler's ``interpolationScheme cell``).
"""

from __future__ import annotations

from typing import Dict, Optional

import numpy as np


def _ascii(a: np.ndarray, fmt: str) -> str:
    return " ".join(fmt % x for x in np.asarray(a).ravel())


def write_vtp(path: str, offsets: np.ndarray, points: np.ndarray, cells: np.ndarray,
              cell_fields: Optional[Dict[str, np.ndarray]] = None) -> None:
    """Write polygons (points[offsets[k]:offsets[k+1]] for polygon k) with
    ``cellIds`` and every field of ``cell_fields`` (indexed by mesh cell,
    scalar or 3-vector) sampled at each polygon's cell."""
    offsets = np.asarray(offsets, dtype=np.int64)
    points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    cells = np.asarray(cells, dtype=np.int64)
    n_poly = cells.size
    if offsets.size != n_poly + 1 or offsets[-1] != points.shape[0]:
        raise ValueError("offsets, points and cells do not describe the same polygons")
    fields = {"cellIds": cells}
    for name, f in (cell_fields or {}).items():
        fields[name] = np.asarray(f)[cells]
    with open(path, "w") as fh:
        fh.write('<?xml version="1.0"?>\n')
        fh.write('<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        fh.write("<PolyData>\n")
        fh.write(f'<Piece NumberOfPoints="{points.shape[0]}" NumberOfVerts="0" NumberOfLines="0" '
                 f'NumberOfStrips="0" NumberOfPolys="{n_poly}">\n')
        fh.write('<Points>\n<DataArray type="Float64" NumberOfComponents="3" format="ascii">\n')
        fh.write(_ascii(points, "%.17g") + "\n</DataArray>\n</Points>\n")
        fh.write("<Polys>\n")
        fh.write('<DataArray type="Int64" Name="connectivity" format="ascii">\n')
        fh.write(_ascii(np.arange(points.shape[0]), "%d") + "\n</DataArray>\n")
        fh.write('<DataArray type="Int64" Name="offsets" format="ascii">\n')
        fh.write(_ascii(offsets[1:], "%d") + "\n</DataArray>\n</Polys>\n")
        fh.write("<CellData>\n")
        for name, v in fields.items():
            v = np.asarray(v)
            comps = 1 if v.ndim == 1 else v.shape[1]
            if np.issubdtype(v.dtype, np.integer):
                fh.write(f'<DataArray type="Int64" Name="{name}" NumberOfComponents="{comps}" format="ascii">\n')
                fh.write(_ascii(v, "%d") + "\n</DataArray>\n")
            else:
                fh.write(f'<DataArray type="Float64" Name="{name}" NumberOfComponents="{comps}" format="ascii">\n')
                fh.write(_ascii(v, "%.17g") + "\n</DataArray>\n")
        fh.write("</CellData>\n</Piece>\n</PolyData>\n</VTKFile>\n")


def read_vtp(path: str):
    """(offsets, points, cell data) of a file written by write_vtp."""
    import xml.etree.ElementTree as ET

    root = ET.parse(path).getroot()
    piece = root.find("PolyData/Piece")
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float64).reshape(-1, 3)
    arrays = {a.get("Name"): a for a in piece.find("Polys").findall("DataArray")}
    off = np.concatenate(([0], np.array(arrays["offsets"].text.split(), dtype=np.int64)))
    data = {}
    for a in piece.find("CellData").findall("DataArray"):
        dt = np.int64 if a.get("type").startswith("Int") else np.float64
        v = np.array(a.text.split(), dtype=dt)
        comps = int(a.get("NumberOfComponents", "1"))
        data[a.get("Name")] = v.reshape(-1, comps) if comps > 1 else v
    return off, pts, data
