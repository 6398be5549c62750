"""VTU output of designs (XML UnstructuredGrid, no third-party writer).

* ``export_mesh_with_info`` mirrors sktopt/core/visualization.py:22-84: the
  mesh with named cell / point data, written with the element connectivity
  exactly as the mesh stores it (the reference hands ``mesh.t.T`` to meshio
  as VTK cells unchanged, so a hexahedron keeps scikit-fem's local order).
* ``export_submesh`` mirrors sktopt/mesh/visualization.py:11-37: the
  elements that are not design elements with rho <= threshold, nodes
  renumbered in sorted order, saved through scikit-fem's writer, which maps
  hexahedra to the VTK node order (``vtk_order=True`` here).

Data arrays are base64 "binary" with a UInt64 byte-count header, Float64 /
Int64 / UInt8, little endian.  ``read_vtu`` reads files of this layout back.
"""
from __future__ import annotations

import base64
import pathlib
import xml.etree.ElementTree as ET

import numpy as np

_VTK_TYPE = {"hex": 12, "tet": 10}
# MeshHex local order (offsets (0,0,0) (0,1,0) (1,0,0) (0,0,1) (1,1,0)
# (0,1,1) (1,0,1) (1,1,1)) -> VTK hexahedron order
_LOCAL_TO_VTK_HEX = [0, 2, 4, 1, 3, 6, 7, 5]
_DT = {np.dtype(np.float64): "Float64", np.dtype(np.int64): "Int64",
       np.dtype(np.uint8): "UInt8", np.dtype(np.float32): "Float32",
       np.dtype(np.int32): "Int32"}


def _b64(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    raw = a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
    return base64.b64encode(np.uint64(len(raw)).tobytes() + raw).decode("ascii")


def _array(name, a, ncomp=1):
    a = np.asarray(a)
    attrs = f'type="{_DT[a.dtype]}"'
    if name:
        attrs += f' Name="{name}"'
    if ncomp > 1:
        attrs += f' NumberOfComponents="{ncomp}"'
    return f'<DataArray {attrs} format="binary">{_b64(a)}</DataArray>'


def write_vtu(path, points, t, kind, cell_data=None, point_data=None, vtk_order=False):
    """points (3, n), t (nloc, n_elem) in the mesh's local order."""
    t = np.asarray(t, dtype=np.int64)
    if kind == "hex" and vtk_order:
        t = t[_LOCAL_TO_VTK_HEX]
    ne, nloc = t.shape[1], t.shape[0]
    parts = ['<?xml version="1.0"?>',
             '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
             'header_type="UInt64">', "<UnstructuredGrid>",
             f'<Piece NumberOfPoints="{points.shape[1]}" NumberOfCells="{ne}">',
             "<Points>", _array(None, np.asarray(points, np.float64).T, 3), "</Points>",
             "<Cells>", _array("connectivity", t.T.ravel()),
             _array("offsets", np.arange(1, ne + 1, dtype=np.int64) * nloc),
             _array("types", np.full(ne, _VTK_TYPE[kind], dtype=np.uint8)), "</Cells>"]
    if point_data:
        parts.append("<PointData>")
        parts += [_array(k, np.asarray(v, np.float64)) for k, v in point_data.items()]
        parts.append("</PointData>")
    if cell_data:
        parts.append("<CellData>")
        parts += [_array(k, np.asarray(v, np.float64)) for k, v in cell_data.items()]
        parts.append("</CellData>")
    parts += ["</Piece>", "</UnstructuredGrid>", "</VTKFile>"]
    pathlib.Path(path).write_text("\n".join(parts) + "\n")


def _decode(el):
    dt = {v: k for k, v in _DT.items()}[el.get("type")]
    raw = base64.b64decode(el.text.strip())
    n = int(np.frombuffer(raw[:8], dtype="<u8")[0])
    a = np.frombuffer(raw[8:8 + n], dtype=dt.newbyteorder("<")).astype(dt)
    k = int(el.get("NumberOfComponents", "1"))
    return a.reshape(-1, k) if k > 1 else a


def read_vtu(path) -> dict:
    """points (3, n), connectivity (nloc, n_elem), types, cell / point data."""
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    pts = _decode(piece.find("Points/DataArray")).T
    cells = {el.get("Name"): _decode(el) for el in piece.findall("Cells/DataArray")}
    nloc = int(cells["offsets"][0]) if cells["offsets"].size else 0
    out = {"points": pts, "types": cells["types"],
           "connectivity": cells["connectivity"].reshape(-1, nloc).T,
           "cell_data": {el.get("Name"): _decode(el)
                         for el in piece.findall("CellData/DataArray")},
           "point_data": {el.get("Name"): _decode(el)
                          for el in piece.findall("PointData/DataArray")}}
    return out


def export_mesh_with_info(mesh, point_data_values=None, point_data_names=None,
                          cell_data_values=None, cell_data_names=None,
                          filepath="output.vtu"):
    """sktopt/core/visualization.py:22-84."""
    if mesh.kind not in _VTK_TYPE:
        raise ValueError(f"Unsupported mesh type: {mesh.kind}")
    pdata = dict(zip(point_data_names, point_data_values)) \
        if point_data_values and point_data_names else None
    cdata = dict(zip(cell_data_names, cell_data_values)) \
        if cell_data_values and cell_data_names else None
    write_vtu(filepath, mesh.p, mesh.t, mesh.kind, cell_data=cdata, point_data=pdata)


def export_submesh(tsk, rho_projected, threshold: float, dst_path: str):
    """sktopt/mesh/visualization.py:11-37."""
    mesh = tsk.mesh
    design = np.asarray(tsk.design_elements)
    remove = design[np.asarray(rho_projected)[design] <= threshold]
    keep = np.setdiff1d(np.arange(mesh.nelements), remove, assume_unique=False)
    kept_t = mesh.t[:, keep]
    verts = np.unique(kept_t)
    remap = np.full(mesh.nnodes, -1, dtype=np.int64)
    remap[verts] = np.arange(verts.size)
    write_vtu(dst_path, mesh.p[:, verts], remap[kept_t], mesh.kind, vtk_order=True)
