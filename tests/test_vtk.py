"""CPU tests of the VTK XML writer (omega3d_gb300/vtk.py, after Points::write_vtk,
Points.h:851-1039): the file parses as XML, carries the reference's arrays with their names
and types, and every array round-trips bit for bit."""
import xml.etree.ElementTree as ET

import numpy as np

import omega3d_gb300 as G
from omega3d_gb300 import vtk


def test_particles_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    n = 257
    x = rng.normal(size=(3, n)).astype(np.float32)
    s = rng.normal(size=(3, n)).astype(np.float32)
    r = rng.uniform(0.01, 0.05, n).astype(np.float32)
    u = rng.normal(size=(3, n)).astype(np.float32)
    ug = rng.normal(size=(9, n)).astype(np.float32)
    p = G.Points(x, s, r, u=u, ug=ug)
    path = vtk.write_vtk(p, 3, 42, 1.25, directory=str(tmp_path), grads=True)
    assert path.endswith("part_03_00042.vtu")
    root = ET.parse(path).getroot()
    assert root.get("type") == "UnstructuredGrid" and root.get("header_type") == "UInt32"
    piece = root.find("UnstructuredGrid/Piece")
    assert piece.get("NumberOfPoints") == str(n) and piece.get("NumberOfCells") == str(n)
    d = vtk.read_vtu(path)
    assert d["TimeValue"][0] == 1.25
    assert np.array_equal(d["position"], x) and np.array_equal(d["circulation"], s)
    assert np.array_equal(d["radius"], r) and np.array_equal(d["velocity"], u)
    assert np.array_equal(d["velocity_gradient"], ug)
    assert np.array_equal(d["connectivity"], np.arange(n)) and np.array_equal(d["offsets"], np.arange(1, n + 1))
    assert np.all(d["types"] == 1)


def test_field_points_have_no_strength_or_radius(tmp_path):
    x = np.zeros((3, 5), np.float32)
    p = G.Points(x, None, None, inert=True)
    path = vtk.write_vtk(p, 0, 7, 0.0, directory=str(tmp_path))
    assert path.endswith("fldpt_00_00007.vtu")
    d = vtk.read_vtu(path)
    assert "circulation" not in d and "radius" not in d and d["velocity"].shape == (3, 5)


def test_surface_vtu_round_trip(tmp_path):
    """Surfaces::write_vtk layout: triangles over the nodes, the vortex sheet vector
    ps0 x1 + ps1 x2 (float) and the source sheet strength as cell data."""
    import omega3d_gb300 as G
    from omega3d_gb300 import vtk
    x, i = G.generate_ovoid(1, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=3)
    rng = np.random.default_rng(4)
    s.set_sheet_strengths(rng.normal(size=s.npanels).astype(np.float32),
                          rng.normal(size=s.npanels).astype(np.float32),
                          rng.normal(size=s.npanels).astype(np.float32))
    path = vtk.write_surface_vtk(s, 1, 12, 0.25, directory=str(tmp_path))
    assert path.endswith("panel_01_00012.vtu")
    d = vtk.read_vtu(path)
    assert np.array_equal(d["position"], s.x)
    assert np.array_equal(d["connectivity"], s.idx.astype(np.int32))
    assert np.array_equal(d["offsets"], 3 * np.arange(1, s.npanels + 1, dtype=np.int32))
    assert np.all(d["types"] == 5)
    sheet = (s.ps[0] * s.x1 + s.ps[1] * s.x2).astype(np.float32)
    assert np.array_equal(d["vortex sheet strength"], sheet)
    assert np.array_equal(d["source sheet strength"], s.ps[2])
    assert d["TimeValue"][0] == 0.25
