"""CPU tests of the library's host-side geometry (sphere, panel bases, sheet strengths):
bit-identical to the oracle's restatement of GeomHelper.cpp / IglRefine.cpp / igl
upsample / Surfaces.h, and to the committed sphere fixture."""
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def G(built_lib):
    import omega3d_gb300
    return omega3d_gb300


@pytest.mark.parametrize("lev", [0, 1, 2, 3, 4, 5])
def test_sphere_matches_oracle_bit_exact(G, lev):
    x, i = G.generate_ovoid(lev, 2.0, 2.0, 2.0)
    xo, io = O.generate_ovoid(lev, 2.0, 2.0, 2.0)
    assert x.shape == (3, 10 * 4 ** lev + 2) and i.shape == (3 * 20 * 4 ** lev,)
    assert np.array_equal(x, xo) and np.array_equal(i, io)
    if lev <= 3:
        d = np.load(os.path.join(GOLD, "sphere.npz"))
        assert np.array_equal(x, d["nodes_L%d" % lev]) and np.array_equal(i, d["idx_L%d" % lev])


def test_bases_and_strengths_match_oracle(G):
    x, i = G.generate_ovoid(3, 2.0, 1.5, 1.0)
    s = G.Surfaces(x, i)
    x1, x2, nm, ar = O.compute_bases(x, i)
    for a, b in ((s.x1, x1), (s.x2, x2), (s.norm, nm), (s.area, ar)):
        assert np.array_equal(a, b)
    rng = np.random.default_rng(9)
    p0 = rng.normal(size=s.npanels).astype(np.float32)
    p1 = rng.normal(size=s.npanels).astype(np.float32)
    s.set_sheet_strengths(p0, p1)
    assert np.array_equal(s.ts, O.sheet_to_panel_strength(p0, p1, x1, x2, ar))
    # orthonormal bases, outward normals on the sphere, areas summing to the surface area
    assert np.allclose((s.x1 * s.x2).sum(0), 0, atol=1e-6)
    assert np.allclose(np.linalg.norm(s.norm, axis=0), 1, atol=1e-6)


def test_unit_sphere_area_and_normals(G):
    x, i = G.generate_ovoid(4, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i)
    assert abs(s.area.sum() - 4 * np.pi) / (4 * np.pi) < 5e-3
    f = i.reshape(-1, 3)
    cen = (x[:, f[:, 0]] + x[:, f[:, 1]] + x[:, f[:, 2]]) / 3
    assert np.all((cen * s.norm).sum(0) > 0)   # x1 x x2 points out of the body


def test_geometry_argument_checks(G):
    lib = G.lib()
    import ctypes
    a, b = ctypes.c_int32(), ctypes.c_int32()
    assert lib.o3g_ovoid_size(-1, ctypes.byref(a), ctypes.byref(b)) == 1
    assert lib.o3g_ovoid_size(5, ctypes.byref(a), ctypes.byref(b)) == 0 and (a.value, b.value) == (10242, 20480)
    bad = np.array([0, 1, 99], np.uint32)
    x = np.zeros((3, 3), np.float32)
    out = [np.zeros(1, np.float32) for _ in range(10)]
    assert lib.o3g_compute_bases(3, *[x[k].ctypes.data for k in range(3)], 1, bad.ctypes.data,
                                 *[o.ctypes.data for o in out]) == 1
