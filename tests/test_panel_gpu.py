"""GPU parity tests of the panel kernels and the BEM coefficient block through the C-ABI.

Subdivision decisions are the reference's (same operation order, no FMA in the test), so
results differ from the reference semantics only by FP32 summation order:
  * panels_affect_points / points_affect_panels vs the oracle (prec 1, float pairs with
    double accumulators) and the golden vectors of the reference build (prec 0):
    per-target relative error <= 1e-5 (metrics.rel_err, floor 1e-6 of the max).
  * panels_on_panels_coeff vs the oracle / golden (prec 0): |dC| <= 1e-5 |C| + 1e-6 max|C|
    elementwise, self-influence diagonal exact.
"""
import os

import numpy as np
import pytest

import oracle as O
import omega3d_gb300 as G
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import rel_err

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _sphere(levels, scale=2.0, seed=5, nunk=3):
    x, i = G.generate_ovoid(levels, scale, scale, scale)
    s = G.Surfaces(x, i, nunk=nunk)
    rng = np.random.default_rng(seed)
    s.set_sheet_strengths(rng.normal(size=s.npanels).astype(np.float32),
                          rng.normal(size=s.npanels).astype(np.float32),
                          rng.normal(size=s.npanels).astype(np.float32))
    return s


def _targets(n, seed, near=0.2):
    tx, ts, tr = W.shell_particles(n, seed=seed, rin=1.0 + near * 0.1, rout=1.6)
    return tx, ts, tr


@pytest.mark.parametrize("grads", [True, False])
@pytest.mark.parametrize("src", [True, False])
@pytest.mark.parametrize("on_device", [True, False])
def test_panels_affect_points_vs_oracle(cuda, grads, src, on_device):
    import torch
    s = _sphere(2, nunk=3 if src else 2)
    tx, _, _ = _targets(700, 11)
    tx[:, :60] *= np.float32(1.0 / 1.08)   # close to the surface: subdivision down to level 3
    uo, go = O.panels_affect_points(s.x, s.idx, s.area, s.ts, tx, s.ps[2] if src else None, grads, "rm", 1)
    if on_device:
        targ = G.Points(torch.from_numpy(tx).cuda(), None, None, inert=True, grads=grads)
        G.panels_affect_points(s, targ, G.ResultsType("velandgrad" if grads else "velonly"),
                               arrays=s.device_arrays("cuda"))
        torch.cuda.synchronize()
        u = targ.u.cpu().numpy()
        g = targ.ug.cpu().numpy() if grads else None
    else:
        targ = G.Points(tx, None, None, inert=True, grads=grads)
        G.panels_affect_points(s, targ, G.ResultsType("velandgrad" if grads else "velonly"))
        u, g = targ.u, targ.ug
    assert rel_err(u, uo)[0] <= 1e-5
    if grads:
        assert rel_err(g, go)[0] <= 1e-5


@pytest.mark.parametrize("core", ["rm", "wl", "exp"])
def test_panel_golden_vectors(cuda, core):
    d = np.load(os.path.join(GOLD, "panel_%s.npz" % core))
    s = G.Surfaces(d["nodes"], d["idx"])
    s.ts[...] = d["ts"]
    s.ps[2] = d["sss"]
    targ = G.Points(np.ascontiguousarray(d["tx"]), None, None, inert=True)
    G.panels_affect_points(s, targ)
    assert rel_err(targ.u, d["pg_u_p0"])[0] <= 1e-5 and rel_err(targ.ug, d["pg_g_p0"])[0] <= 1e-5
    assert rel_err(targ.u, d["pg_u_p2"])[0] <= 1e-5
    src = G.Points(np.ascontiguousarray(d["tx"]), np.ascontiguousarray(d["ps"]), np.ones(d["tx"].shape[1], np.float32))
    s.pu[...] = 0
    G.points_affect_panels(src, s)
    assert rel_err(s.pu, d["pan_u_p0"])[0] <= 1e-5


@pytest.mark.parametrize("on_device", [True, False])
def test_points_affect_panels_vs_oracle(cuda, on_device):
    import torch
    s = _sphere(3)
    px, ps, pr = _targets(3000, 12)
    px[:, :100] *= np.float32(1.0 / 1.1)
    po = O.points_affect_panels(px, ps, s.x, s.idx, s.area, "rm", 1)
    src_np = G.Points(px, ps, pr)
    if on_device:
        arr = s.device_arrays("cuda")
        src = G.Points(*(torch.from_numpy(a).cuda() for a in (px, ps, pr)))
        pu = torch.zeros(3, s.npanels, device="cuda")
        G.points_affect_panels(src, s, arrays=arr, pu=pu)
        torch.cuda.synchronize()
        got = pu.cpu().numpy()
    else:
        s.pu[...] = 0
        G.points_affect_panels(src_np, s)
        got = s.pu
    assert rel_err(got, po)[0] <= 1e-5


def _coeff_gpu(s, nunk, maxlev=3):
    import torch
    arr = s.device_arrays("cuda")
    n = s.npanels * nunk
    out = torch.full((n, n), float("nan"), device="cuda")   # every entry must be written
    G.panels_on_panels_coeff(arr, arr, nunk, True, out, maxlev=maxlev)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _close(c, ref):
    scale = np.abs(ref).max()
    return np.all(np.abs(c - ref) <= 1e-5 * np.abs(ref) + 1e-6 * scale)


@pytest.mark.parametrize("nunk", [2, 3])
def test_coefficients_vs_golden(cuda, nunk):
    d = np.load(os.path.join(GOLD, "coeff_rm.npz"))
    s = G.Surfaces(d["nodes"], d["idx"], nunk=nunk)
    c = _coeff_gpu(s, nunk)
    ref = d["c%d_p0" % nunk]
    assert np.all(np.isfinite(c))
    assert _close(c, ref)
    # self-influence diagonal blocks are the reference's constants exactly
    n = s.npanels
    for j in range(0, n, 7):
        blk = c[j * nunk:(j + 1) * nunk, j * nunk:(j + 1) * nunk]
        assert np.array_equal(blk, ref[j * nunk:(j + 1) * nunk, j * nunk:(j + 1) * nunk])


@pytest.mark.parametrize("nunk", [2, 3])
def test_coefficients_vs_oracle_level2(cuda, nunk):
    s = _sphere(2, nunk=nunk)
    geo = dict(nodes=s.x, idx=s.idx, area=s.area, x1=s.x1, x2=s.x2, norm=s.norm)
    ref = O.panels_on_panels_coeff(geo, geo, nunk, True, "rm", 0)
    c = _coeff_gpu(s, nunk)
    assert _close(c, ref)
    # maxlev 0 (no subdivision) is the plain centroid rule
    ref0 = O.panels_on_panels_coeff(geo, geo, nunk, True, "rm", 0, maxlev=0)
    assert _close(_coeff_gpu(s, nunk, maxlev=0), ref0)


def test_coefficient_block_into_larger_matrix(cuda):
    import torch
    s = _sphere(1, nunk=2)
    arr = s.device_arrays("cuda")
    n = s.npanels * 2
    big = torch.zeros((n + 5, 3 * n), device="cuda")         # rows = leading dimension (column-major view)
    G.panels_on_panels_coeff(arr, arr, 2, True, big.view(-1)[(n + 5) * 7 + 3:], ld=n + 5)
    torch.cuda.synchronize()
    ref = _coeff_gpu(s, 2)
    bm = big.cpu().numpy().reshape(-1)
    got = np.stack([bm[(n + 5) * (7 + j) + 3:(n + 5) * (7 + j) + 3 + n] for j in range(n)])
    assert np.array_equal(got, ref)


def _collocation(s):
    """Surfaces::represent_as_particles(0.0001, ...) positions (Surfaces.h:991-997) in the
    reference's float arithmetic: (1/3 in double) * (float sum), then + offset * normal."""
    i = s.idx.reshape(-1, 3)
    tot = (s.x[:, i[:, 0]] + s.x[:, i[:, 1]]) + s.x[:, i[:, 2]]
    c = (np.float64(1.0 / 3.0) * tot.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(c + np.float32(0.0001) * s.norm)


@pytest.mark.parametrize("on_device", [True, False])
@pytest.mark.parametrize("self_influence", [True, False])
def test_panels_affect_panels_vs_oracle(cuda, on_device, self_influence):
    """Influence.h:1223-1243: velocity of the source panels at the target panels'
    collocation points, written (not accumulated) into the target's panel velocities."""
    import torch
    s = _sphere(2, nunk=3)
    t = s if self_influence else _sphere(1, scale=3.2, seed=6, nunk=2)
    pts = _collocation(t)
    uo, _ = O.panels_affect_points(s.x, s.idx, s.area, s.ts, pts, s.ps[2], False, "rm", 1)
    if on_device:
        sa, ta = s.device_arrays("cuda"), t.device_arrays("cuda")
        pu = torch.full((3, t.npanels), 7.0, device="cuda")
        G.panels_affect_panels(s, t, src_arrays=sa, targ_arrays=ta, pu=pu)
        torch.cuda.synchronize()
        u = pu.cpu().numpy()
    else:
        t.pu[...] = 7.0
        G.InfluenceVisitor(G.ResultsType("velonly"))(s, t)
        u = t.pu.copy()
    assert rel_err(u, uo)[0] <= 1e-5
    assert np.abs(u).max() > 0


def test_centroid_division_by_three_is_ieee_for_every_float(cuda):
    """The panel kernels form centroids as (a + b + c) / 3 in the reference's float order;
    the division is a multiply by RN(1/3) and one fma correction (Markstein).  It must give
    the IEEE quotient, bit for bit, for every one of the 2^32 float inputs."""
    import ctypes
    from omega3d_gb300 import _lib as L
    bad = ctypes.c_uint64(1)
    assert L.lib().o3g_div3_check(0, 1 << 32, ctypes.byref(bad), None) == 0
    assert bad.value == 0
