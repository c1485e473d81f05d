"""VTK XML output of particle and field-point sets, as Points::write_vtk writes them, and of
panel surfaces, as Surfaces::write_vtk writes them
(Points.h:851-1039, VtkXmlWriter.h): an UnstructuredGrid of vertex cells with the
simulation time as FieldData "TimeValue", Float32 "position", Int32 "connectivity" and
"offsets", UInt8 "types" (1 = vertex), and PointData "circulation" (3 components, active
particles only), "radius" (active particles only) and "velocity" (3 components); the
optional "velocity_gradient" (9 components, the reference's order) is this library's
addition.  Arrays are base64 "binary" blocks preceded by a UInt32 byte count.  The length
block holds the number of data bytes, as the VTK format specifies; the reference's writer
stores the length of the encoded text there instead (VtkXmlWriter.h:97-100).

File names follow the reference: part_<index:02>_<frame:05>.vtu for particles,
fldpt_<index:02>_<frame:05>.vtu for field points and panel_<index:02>_<frame:05>.vtu for
surfaces.
"""
import base64
import os
import struct

import numpy as np


def _host(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except Exception:  # pragma: no cover
        pass
    return np.asarray(a)


def _block(arr):
    raw = np.ascontiguousarray(arr).tobytes()
    return base64.b64encode(struct.pack("<I", len(raw))).decode() + base64.b64encode(raw).decode()


def _interleave(a):
    a = _host(a)
    if a.ndim == 1:
        return a.astype(np.float32)
    k, n = a.shape
    out = np.zeros((n, 3 if k <= 3 else k), np.float32)
    out[:, :k] = a.T
    return out.reshape(-1)


def _array(name, typ, data, ncomp=None):
    attrs = 'Name="%s" type="%s"' % (name, typ)
    if ncomp:
        attrs = 'Name="%s" NumberOfComponents="%d" type="%s"' % (name, ncomp, typ)
    return '<DataArray %s format="binary">\n %s \n</DataArray>\n' % (attrs, _block(data))


def write_points_vtu(path, x, u=None, s=None, r=None, ug=None, time=0.0):
    """Writes one points file.  x: positions [3, n]; u: velocities [3, n]; s: strengths
    [3, n] and r: radii [n] (active particles; omit both for field points); ug: gradients
    [9, n] (optional).  Numpy arrays or torch tensors.  Returns the path."""
    xh = _host(x)
    n = xh.shape[1]
    parts = ['<?xml version="1.0" encoding="UTF-8"?>\n',
             '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" header_type="UInt32">\n',
             '<UnstructuredGrid>\n<FieldData>\n',
             _array("TimeValue", "Float64", np.array([time], np.float64)).replace(
                 'Name="TimeValue" type="Float64"', 'Name="TimeValue" NumberOfTuples="1" type="Float64"'),
             '</FieldData>\n<Piece NumberOfCells="%d" NumberOfPoints="%d">\n<Points>\n' % (n, n),
             _array("position", "Float32", _interleave(xh), 3),
             '</Points>\n<Cells>\n',
             _array("connectivity", "Int32", np.arange(n, dtype=np.int32)),
             _array("offsets", "Int32", np.arange(1, n + 1, dtype=np.int32)),
             _array("types", "UInt8", np.ones(n, np.uint8)),
             '</Cells>\n']
    scal = ' Scalars="radius"' if r is not None else ''
    parts.append('<PointData%s Vectors="velocity">\n' % scal)
    if s is not None:
        parts.append(_array("circulation", "Float32", _interleave(s), 3))
    if r is not None:
        parts.append(_array("radius", "Float32", _host(r).astype(np.float32)))
    parts.append(_array("velocity", "Float32", _interleave(u if u is not None else np.zeros((3, n), np.float32)), 3))
    if ug is not None:
        parts.append(_array("velocity_gradient", "Float32", _interleave(ug), 9))
    parts.append('</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n')
    with open(path, "w") as f:
        f.write("".join(parts))
    return path


def write_vtk(points, index, frameno, time, directory=".", grads=False):
    """Points::write_vtk naming: part_II_FFFFF.vtu (active) or fldpt_II_FFFFF.vtu (inert)."""
    prefix = "fldpt_" if points.inert else "part_"
    path = os.path.join(directory, "%s%02d_%05d.vtu" % (prefix, index, frameno))
    return write_points_vtu(path, points.x, points.u, None if points.inert else points.s,
                            None if points.inert else points.r, points.ug if grads else None, time)


def write_surface_vtu(path, nodes, idx, sheet=None, src=None, time=0.0):
    """Writes one panel file as Surfaces::write_vtk does (Surfaces.h:1301-1458): an
    UnstructuredGrid of triangles (type 5) over the nodes [3, nn], Float32 "position",
    Int32 "connectivity" (idx) and "offsets" (3, 6, ...), and CellData "vortex sheet
    strength" (3 components per panel) and "source sheet strength" (scalar) when given.
    Returns the path."""
    xh = _host(nodes)
    ih = _host(idx).astype(np.int64).reshape(-1)
    nn, npan = xh.shape[1], ih.size // 3
    parts = ['<?xml version="1.0" encoding="UTF-8"?>\n',
             '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" header_type="UInt32">\n',
             '<UnstructuredGrid>\n<FieldData>\n',
             _array("TimeValue", "Float64", np.array([time], np.float64)).replace(
                 'Name="TimeValue" type="Float64"', 'Name="TimeValue" NumberOfTuples="1" type="Float64"'),
             '</FieldData>\n<Piece NumberOfCells="%d" NumberOfPoints="%d">\n<Points>\n' % (npan, nn),
             _array("position", "Float32", _interleave(xh), 3),
             '</Points>\n<Cells>\n',
             _array("connectivity", "Int32", ih.astype(np.int32)),
             _array("offsets", "Int32", (3 * np.arange(1, npan + 1)).astype(np.int32)),
             _array("types", "UInt8", np.full(npan, 5, np.uint8)),
             '</Cells>\n']
    if sheet is not None or src is not None:
        attrs = ''
        if src is not None:
            attrs += ' Scalars="source sheet strength"'
        if sheet is not None:
            attrs += ' Vectors="vortex sheet strength"'
        parts.append('<CellData%s>\n' % attrs)
        if sheet is not None:
            parts.append(_array("vortex sheet strength", "Float32", _interleave(sheet), 3))
        if src is not None:
            parts.append(_array("source sheet strength", "Float32", _host(src).astype(np.float32)))
        parts.append('</CellData>\n')
    parts.append('</Piece>\n</UnstructuredGrid>\n</VTKFile>\n')
    with open(path, "w") as f:
        f.write("".join(parts))
    return path


def sheet_vectors(surf):
    """Surfaces::vortex_sheet_to_vector (Surfaces.h:340-361) in float: ps0 x1 + ps1 x2."""
    ps0, ps1 = surf.ps[0].astype(np.float32), surf.ps[1].astype(np.float32)
    return (ps0 * surf.x1 + ps1 * surf.x2).astype(np.float32)


def write_surface_vtk(surf, index, frameno, time, directory="."):
    """Surfaces::write_vtk naming: panel_II_FFFFF.vtu, with the vortex sheet strength and,
    for three unknowns per panel, the source sheet strength."""
    path = os.path.join(directory, "panel_%02d_%05d.vtu" % (index, frameno))
    return write_surface_vtu(path, surf.x, surf.idx, sheet_vectors(surf), surf.ps[2] if surf.nunk == 3 else None,
                             time)


def read_vtu(path):
    """Reads a file written by write_points_vtu back into {name: array} (for tests/tools)."""
    import xml.etree.ElementTree as ET
    root = ET.parse(path).getroot()
    types = {"Float32": np.float32, "Float64": np.float64, "Int32": np.int32, "UInt8": np.uint8}
    out = {}
    for da in root.iter("DataArray"):
        text = "".join(da.text.split())
        head = base64.b64decode(text[:8])
        nbytes = struct.unpack("<I", head)[0]
        raw = base64.b64decode(text[8:])
        assert len(raw) == nbytes
        a = np.frombuffer(raw, dtype=types[da.get("type")])
        nc = int(da.get("NumberOfComponents", "1"))
        out[da.get("Name")] = a.reshape(-1, nc).T.copy() if nc > 1 else a.copy()
    return out
