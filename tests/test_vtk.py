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
