"""VTK XML output of particle and field-point sets, as Points::write_vtk writes them, and of
panel surfaces, as Surfaces::write_vtk writes them
(Points.h:851-1039, Surfaces.h:1301-1458, VtkXmlWriter.h): an UnstructuredGrid of vertex
cells (particles) or triangles (panels) with the simulation time as FieldData "TimeValue",
Float32 "position", Int32 "connectivity" and "offsets", UInt8 "types", and PointData
"circulation" (3 components, active particles only), "radius" (active particles only) and
"velocity" (3 components), or CellData "vortex sheet strength" and "source sheet strength";
the optional "velocity_gradient" (9 components, the reference's order) is this library's
addition.

Arrays are base64 "binary" blocks, each a base64 UInt32 length block followed by the
base64 data.  By default (length_header="reference") the files are byte for byte those of
the reference's writer: its XML layout (tinyxml2's printer: the `<?xml version="1.0"?>`
declaration, four spaces of indentation per level, data inline between single spaces)
and its length block, which holds the length of the encoded text (VtkXmlWriter.h:97-100).
length_header="vtk" stores the number of data bytes there instead, as the VTK format
specifies.  read_vtu reads both.

File names follow the reference: part_<index:02>_<frame:05>.vtu for particles,
fldpt_<index:02>_<frame:05>.vtu for field points and panel_<index:02>_<frame:05>.vtu for
surfaces.
"""
import base64
import os
import struct

import numpy as np

HEADERS = ("reference", "vtk")


def _host(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except Exception:  # pragma: no cover
        pass
    return np.asarray(a)


def _block(arr, length_header):
    raw = np.ascontiguousarray(arr).tobytes()
    data = base64.b64encode(raw)
    length = len(data) if length_header == "reference" else len(raw)
    return base64.b64encode(struct.pack("<I", length)).decode() + data.decode()


def _interleave(a):
    a = _host(a)
    if a.ndim == 1:
        return a.astype(np.float32)
    k, n = a.shape
    out = np.zeros((n, 3 if k <= 3 else k), np.float32)
    out[:, :k] = a.T
    return out.reshape(-1)


class _Printer:
    """The subset of tinyxml2's XMLPrinter layout the reference's files use: one element per
    line, indented four spaces per level; a data array's text on its element's line."""

    def __init__(self):
        self.out = ['<?xml version="1.0"?>\n']
        self.depth = 0

    def open(self, name, attrs=()):
        a = "".join(' %s="%s"' % kv for kv in attrs)
        self.out.append("    " * self.depth + "<%s%s>\n" % (name, a))
        self.depth += 1

    def close(self, name):
        self.depth -= 1
        self.out.append("    " * self.depth + "</%s>\n" % name)

    def data(self, attrs, block):
        a = "".join(' %s="%s"' % kv for kv in attrs)
        self.out.append("    " * self.depth + '<DataArray%s format="binary"> %s </DataArray>\n' % (a, block))

    def text(self):
        return "".join(self.out)


def _array(pr, name, typ, data, length_header, ncomp=None, tuples=None):
    # attributes in the order of the reference's std::map: Name, NumberOf..., type
    attrs = [("Name", name)]
    if ncomp:
        attrs.append(("NumberOfComponents", str(ncomp)))
    if tuples:
        attrs.append(("NumberOfTuples", str(tuples)))
    attrs.append(("type", typ))
    pr.data(attrs, _block(data, length_header))


def _head(pr, time, npts, ncells, length_header):
    pr.open("VTKFile", [("type", "UnstructuredGrid"), ("version", "0.1"), ("byte_order", "LittleEndian"),
                        ("header_type", "UInt32")])
    pr.open("UnstructuredGrid")
    pr.open("FieldData")
    _array(pr, "TimeValue", "Float64", np.array([time], np.float64), length_header, tuples=1)
    pr.close("FieldData")
    pr.open("Piece", [("NumberOfCells", str(ncells)), ("NumberOfPoints", str(npts))])


def _tail(pr):
    pr.close("Piece")
    pr.close("UnstructuredGrid")
    pr.close("VTKFile")


def write_points_vtu(path, x, u=None, s=None, r=None, ug=None, time=0.0, length_header="reference"):
    """Writes one points file.  x: positions [3, n]; u: velocities [3, n]; s: strengths
    [3, n] and r: radii [n] (active particles; omit both for field points); ug: gradients
    [9, n] (optional).  Numpy arrays or torch tensors.  Returns the path."""
    if length_header not in HEADERS:
        raise ValueError("length_header must be one of %s" % (HEADERS,))
    xh = _host(x)
    n = xh.shape[1]
    pr = _Printer()
    _head(pr, time, n, n, length_header)
    pr.open("Points")
    _array(pr, "position", "Float32", _interleave(xh), length_header, ncomp=3)
    pr.close("Points")
    pr.open("Cells")
    _array(pr, "connectivity", "Int32", np.arange(n, dtype=np.int32), length_header)
    _array(pr, "offsets", "Int32", np.arange(1, n + 1, dtype=np.int32), length_header)
    _array(pr, "types", "UInt8", np.ones(n, np.uint8), length_header)
    pr.close("Cells")
    pr.open("PointData", ([("Scalars", "radius")] if r is not None else []) + [("Vectors", "velocity")])
    if s is not None:
        _array(pr, "circulation", "Float32", _interleave(s), length_header, ncomp=3)
    if r is not None:
        _array(pr, "radius", "Float32", _host(r).astype(np.float32), length_header)
    _array(pr, "velocity", "Float32", _interleave(u if u is not None else np.zeros((3, n), np.float32)), length_header,
           ncomp=3)
    if ug is not None:
        _array(pr, "velocity_gradient", "Float32", _interleave(ug), length_header, ncomp=9)
    pr.close("PointData")
    _tail(pr)
    with open(path, "w") as f:
        f.write(pr.text())
    return path


def write_vtk(points, index, frameno, time, directory=".", grads=False, length_header="reference"):
    """Points::write_vtk naming: part_II_FFFFF.vtu (active) or fldpt_II_FFFFF.vtu (inert)."""
    prefix = "fldpt_" if points.inert else "part_"
    path = os.path.join(directory, "%s%02d_%05d.vtu" % (prefix, index, frameno))
    return write_points_vtu(path, points.x, points.u, None if points.inert else points.s,
                            None if points.inert else points.r, points.ug if grads else None, time, length_header)


def write_surface_vtu(path, nodes, idx, sheet=None, src=None, time=0.0, length_header="reference"):
    """Writes one panel file as Surfaces::write_vtk does (Surfaces.h:1301-1458): an
    UnstructuredGrid of triangles (type 5) over the nodes [3, nn], Float32 "position",
    Int32 "connectivity" (idx) and "offsets" (3, 6, ...), and CellData "vortex sheet
    strength" (3 components per panel) and "source sheet strength" (scalar) when given
    (the CellData element names the scalars only, as the reference's does).  Returns the
    path."""
    if length_header not in HEADERS:
        raise ValueError("length_header must be one of %s" % (HEADERS,))
    xh = _host(nodes)
    ih = _host(idx).astype(np.int64).reshape(-1)
    nn, npan = xh.shape[1], ih.size // 3
    pr = _Printer()
    _head(pr, time, nn, npan, length_header)
    pr.open("Points")
    _array(pr, "position", "Float32", _interleave(xh), length_header, ncomp=3)
    pr.close("Points")
    pr.open("Cells")
    _array(pr, "connectivity", "Int32", ih.astype(np.int32), length_header)
    _array(pr, "offsets", "Int32", (3 * np.arange(1, npan + 1)).astype(np.int32), length_header)
    _array(pr, "types", "UInt8", np.full(npan, 5, np.uint8), length_header)
    pr.close("Cells")
    if sheet is not None or src is not None:
        pr.open("CellData", [("Scalars", "source sheet strength")] if src is not None else [])
        if sheet is not None:
            _array(pr, "vortex sheet strength", "Float32", _interleave(sheet), length_header, ncomp=3)
        if src is not None:
            _array(pr, "source sheet strength", "Float32", _host(src).astype(np.float32), length_header)
        pr.close("CellData")
    _tail(pr)
    with open(path, "w") as f:
        f.write(pr.text())
    return path


def sheet_vectors(surf):
    """Surfaces::vortex_sheet_to_vector (Surfaces.h:340-361) in float: ps0 x1 + ps1 x2."""
    ps0, ps1 = surf.ps[0].astype(np.float32), surf.ps[1].astype(np.float32)
    return (ps0 * surf.x1 + ps1 * surf.x2).astype(np.float32)


def write_surface_vtk(surf, index, frameno, time, directory=".", length_header="reference"):
    """Surfaces::write_vtk naming: panel_II_FFFFF.vtu, with the vortex sheet strength and,
    for three unknowns per panel, the source sheet strength."""
    path = os.path.join(directory, "panel_%02d_%05d.vtu" % (index, frameno))
    return write_surface_vtu(path, surf.x, surf.idx, sheet_vectors(surf), surf.ps[2] if surf.nunk == 3 else None,
                             time, length_header)


def read_vtu(path):
    """Reads a file written by write_points_vtu / write_surface_vtu (either length header)
    back into {name: array}; the data is the base64 text after the 8-character length block."""
    import xml.etree.ElementTree as ET
    root = ET.parse(path).getroot()
    types = {"Float32": np.float32, "Float64": np.float64, "Int32": np.int32, "UInt8": np.uint8}
    out = {}
    for da in root.iter("DataArray"):
        text = "".join(da.text.split())
        head = struct.unpack("<I", base64.b64decode(text[:8]))[0]
        raw = base64.b64decode(text[8:])
        assert head in (len(raw), len(text) - 8)
        a = np.frombuffer(raw, dtype=types[da.get("type")])
        nc = int(da.get("NumberOfComponents", "1"))
        out[da.get("Name")] = a.reshape(-1, nc).T.copy() if nc > 1 else a.copy()
    return out
