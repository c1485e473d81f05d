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


def _gold():
    import json
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vtk_files.npz"))
    return d, json.loads(str(d["meta"]))


def test_files_are_the_reference_writers_bytes(tmp_path):
    """Particles, field points and panels (with and without the source sheet strength) as
    the reference's own VtkXmlWriter writes them (tests/golden/vtk_files.npz, from the
    reference build), byte for byte: layout, attributes, and the length blocks holding the
    encoded length (VtkXmlWriter.h:97-100)."""
    d, meta = _gold()
    t = meta["times"]
    f = str(tmp_path / "f.vtu")
    cases = (("part", lambda: vtk.write_points_vtu(f, d["x"], d["u"], d["s"], d["r"], time=t["part"])),
             ("fldpt", lambda: vtk.write_points_vtu(f, d["fx"], d["fu"], time=t["fldpt"])),
             ("panel3", lambda: vtk.write_surface_vtu(f, d["nodes"], d["idx"], d["sheet"], d["src"], t["panel3"])),
             ("panel2", lambda: vtk.write_surface_vtu(f, d["nodes"], d["idx"], d["sheet"], None, t["panel2"])))
    for name, call in cases:
        call()
        assert open(f, "rb").read() == d[name].tobytes(), name
        back = vtk.read_vtu(f)
        assert np.array_equal(back["position"], d["x"] if name == "part" else d["fx"] if name == "fldpt" else d["nodes"])


def test_vtk_length_header_mode(tmp_path):
    """length_header="vtk" stores the data's byte count (the VTK format's meaning); the
    files read back the same."""
    import base64
    import struct
    d, _ = _gold()
    a = vtk.write_points_vtu(str(tmp_path / "a.vtu"), d["x"], d["u"], d["s"], d["r"], length_header="vtk")
    root = ET.parse(a).getroot()
    for da in root.iter("DataArray"):
        text = da.text.strip()
        n = struct.unpack("<I", base64.b64decode(text[:8]))[0]
        assert n == len(base64.b64decode(text[8:]))
    b = vtk.read_vtu(a)
    assert np.array_equal(b["circulation"], d["s"]) and np.array_equal(b["radius"], d["r"])


def test_against_the_reference_writer_when_built(tmp_path):
    """Random sizes against the reference build itself (oracle/_ref, when the reference
    sources were there to build it)."""
    import pytest
    import oracle as O
    if not O.ref_vtk_available():
        pytest.skip("oracle/_ref/libo3dref_vtk.so not built (reference sources absent)")
    rng = np.random.default_rng(9)
    for n in (1, 2, 3, 100, 1001):
        x, s, u = (rng.normal(size=(3, n)).astype(np.float32) for _ in range(3))
        r = rng.uniform(0.01, 0.05, n).astype(np.float32)
        a, b = str(tmp_path / "a.vtu"), str(tmp_path / "b.vtu")
        O.ref_write_points_vtu(a, x, u, s, r, 0.5 * n)
        vtk.write_points_vtu(b, x, u, s, r, time=0.5 * n)
        assert open(a, "rb").read() == open(b, "rb").read()
        O.ref_write_points_vtu(a, x, u, None, None, 3.0)
        vtk.write_points_vtu(b, x, u, time=3.0)
        assert open(a, "rb").read() == open(b, "rb").read()
    for lev in (0, 2):
        nodes, idx = O.generate_ovoid(lev, 2.0, 1.0, 0.5)
        npan = idx.size // 3
        sh = rng.normal(size=(3, npan)).astype(np.float32)
        src = rng.normal(size=npan).astype(np.float32)
        a, b = str(tmp_path / "a.vtu"), str(tmp_path / "b.vtu")
        O.ref_write_panels_vtu(a, nodes, idx, sh, src, 7.0)
        vtk.write_surface_vtu(b, nodes, idx, sh, src, 7.0)
        assert open(a, "rb").read() == open(b, "rb").read()
