"""GPU tests of the coupled particle + body path: the compensated panel kernels, and Ralston
RK2 steps whose stages re-solve the BEM of a fixed sphere (o3g_rk2_attach_body) against
the oracle's restatement of Convection::advect_2nd_ralston with solve_bem.

Tolerances:
  * COMPENSATED panel sums vs the oracle with FP32 pair terms and double accumulation
    (prec 1, the reference's subdivision decisions): L-infinity <= 1e-6 (targets 0.01 from
    the sheet, where single FP32 pair terms cancel strongly) and per target <= 1e-5; the
    PLAIN sums of the same inputs are checked at the parity bound 1e-5.
  * one coupled step vs the oracle (prec 1 sums, FP64 LU of the oracle's own matrix):
    particle displacements per particle <= 1e-4 relative, strength changes L-infinity
    <= 1e-4, the stage-2 BEM solution <= 1e-4 relative to its largest entry (the GPU matrix
    differs from the oracle's FP32 one by summation order, <= 1e-5 elementwise).
  * clear_inner_layer: bit-identical to the reference's Reflect.h (golden) and the oracle.
  * with ips > 0 the coupled step also pushes particles out of the body after both moves.
  * potential flow around the sphere from tracer particles (zero strength): RMS error of
    the velocity <= 2e-2 of the freestream at radius 1.3-1.6 (discretisation of 1,280 panels).
"""
import numpy as np
import pytest

import oracle as O
import omega3d_gb300 as G
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import linf_err, rel_err

pytestmark = pytest.mark.gpu


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _sphere(levels, nunk, seed=5):
    x, i = G.generate_ovoid(levels, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=nunk)
    rng = np.random.default_rng(seed)
    s.set_sheet_strengths(rng.normal(size=s.npanels).astype(np.float32),
                          rng.normal(size=s.npanels).astype(np.float32),
                          rng.normal(size=s.npanels).astype(np.float32))
    return s


def test_compensated_panel_sums(cuda):
    import torch
    s = _sphere(3, 3)
    tx, ts_, tr = W.shell_particles(4000, seed=21, rin=1.01, rout=1.8)
    arr = s.device_arrays("cuda")
    for grads in (True, False):
        uo, go = O.panels_affect_points(s.x, s.idx, s.area, s.ts, tx, s.ps[2], grads, "rm", 1)
        for prec in ("compensated", "plain"):
            targ = G.Points(_t(tx), None, None, inert=True, grads=grads)
            G.panels_affect_points(s, targ, G.ResultsType("velandgrad" if grads else "velonly"),
                                   G.ExecEnv("rm", prec), arrays=arr)
            torch.cuda.synchronize()
            u = targ.u.cpu().numpy()
            assert rel_err(u, uo)[0] <= 1e-5
            if prec == "compensated":
                assert linf_err(u, uo) <= 1e-6
            if grads:
                g = targ.ug.cpu().numpy()
                assert rel_err(g, go)[0] <= 1e-5
                if prec == "compensated":
                    assert linf_err(g, go) <= 1e-6
    # points_affect_panels over many particles: the sums run over every particle
    px, ps, pr = W.shell_particles(30000, seed=22, rin=1.01, rout=2.0)
    po = O.points_affect_panels(px, ps, s.x, s.idx, s.area, "rm", 1)
    src = G.Points(_t(px), _t(ps), _t(pr))
    errs = {}
    for prec in ("compensated", "plain"):
        pu = torch.zeros(3, s.npanels, device="cuda")
        G.points_affect_panels(src, s, G.ExecEnv("rm", prec), arrays=arr, pu=pu)
        torch.cuda.synchronize()
        got = pu.cpu().numpy()
        assert rel_err(got, po)[0] <= 1e-5
        errs[prec] = linf_err(got, po)
    assert errs["compensated"] <= 1e-6


def _body(s):
    return dict(nodes=s.x, idx=s.idx, area=s.area, x1=s.x1, x2=s.x2, norm=s.norm)


def _particles(n, seed):
    rng = np.random.default_rng(seed)
    a = W.shell_particles(n // 2, seed=seed, rin=1.03, rout=1.4, sigma=0.02)
    b = W.wake_particles(n - n // 2, seed=seed + 1, xmin=1.0, xmax=2.5, half=0.8, sigma=0.015)
    x = np.concatenate([a[0], b[0]], axis=1)
    s = np.concatenate([a[1], b[1]], axis=1) * np.float32(20.0)
    r = np.concatenate([a[2], b[2]])
    return x, s.astype(np.float32), r, rng


def test_clear_inner_layer_bit_exact(cuda):
    import json
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reflect.npz"))
    ips = json.loads(str(d["meta"]))["ips"]
    x1, x2, nm, area = O.compute_bases(d["nodes"], d["idx"])
    s = G.Surfaces(d["nodes"], d["idx"], nunk=2)
    arr = s.device_arrays("cuda")
    X = _t(d["x_in"])
    n = G.clear_inner_layer(s, G.Points(X, None, None, inert=True), ips=ips, arrays=arr)
    assert n == int(d["npushed_p0"])
    assert np.array_equal(X.cpu().numpy(), d["x_p0"])
    # a larger case against the oracle
    s3 = _sphere(3, 2)
    rng = np.random.default_rng(12)
    v = rng.normal(size=(3, 50000))
    v /= np.linalg.norm(v, axis=0)
    pts = (v * rng.uniform(0.9, 1.1, 50000)).astype(np.float32)
    ref = pts.copy()
    no = O.clear_inner_layer(ref, s3.x, s3.idx, s3.norm, ips=0.02)
    X = _t(pts)
    ng = G.clear_inner_layer(s3, G.Points(X, None, None, inert=True), ips=0.02)
    assert ng == no and np.array_equal(X.cpu().numpy(), ref)


@pytest.mark.parametrize("nunk,ips", [(2, 0.0), (3, 0.0), (2, 0.03)])
def test_coupled_ralston_step_vs_oracle(cuda, nunk, ips):
    import torch
    s = _sphere(2, nunk)
    x, sv, r, _ = _particles(2400, 31)
    if ips > 0:
        x[:, :200] *= np.float32(0.8)       # about half of these inside the body: pushed out
    e = np.ones(x.shape[1], np.float32)
    dt, fs = 0.005, (1.0, 0.0, 0.0)
    X, S, R, E = _t(x), _t(sv), _t(r), _t(e)
    rk = G.Ralston(X, S, R, E, env=G.ExecEnv("rm", "compensated"))
    bem = G.BEM(s.npanels * nunk)
    rk.attach_body(s, bem, ips=ips)
    rk.step(dt, fs, 1)
    torch.cuda.synchronize()
    st = rk.body_stats()
    assert st["solves"] == 2 and st["max_relres"] <= 1e-10
    assert (st["pushed"] > 0) == (ips > 0)
    _, sol_gpu = rk.body_strengths()
    geo = _body(s)
    A = O.panels_on_panels_coeff(geo, geo, nunk, True, "rm", 0).T.astype(np.float64)
    xo, so, eo, sol_o = O.coupled_ralston_step(x, sv, r, e, geo, A, nunk, dt, fs, "rm", 1, ips=ips)
    Xg, Sg, Eg = X.cpu().numpy(), S.cpu().numpy(), E.cpu().numpy()
    assert rel_err(Xg - x, xo - x)[0] <= 1e-4
    assert linf_err(Sg - sv, so - sv) <= 1e-4
    assert np.abs(Eg - eo).max() <= 1e-4 * max(np.abs(eo - 1).max(), 1e-6) + 1e-6
    assert np.abs(sol_gpu - sol_o).max() <= 1e-4 * np.abs(sol_o).max()
    # the body turned the flow: without it the particles move differently
    rk0 = G.Ralston(_t(x), _t(sv), R, _t(e), env=G.ExecEnv("rm", "compensated"), use_graph=False)
    rk0.step(dt, fs, 1)
    torch.cuda.synchronize()
    assert linf_err(rk0.x.cpu().numpy() - x, Xg - x) > 1e-3


def test_tracers_follow_potential_flow_around_sphere(cuda):
    import torch
    s = _sphere(3, 2)
    rng = np.random.default_rng(7)
    n = 2000
    d = rng.normal(size=(3, n))
    d /= np.linalg.norm(d, axis=0)
    x = (d * rng.uniform(1.3, 1.6, n)).astype(np.float32)
    sv = np.zeros((3, n), np.float32)
    r = np.full(n, 0.02, np.float32)
    X = _t(x)
    rk = G.Ralston(X, _t(sv), _t(r), _t(np.ones(n, np.float32)), env=G.ExecEnv("rm", "compensated"))
    bem = G.BEM(s.npanels * 2)
    rk.attach_body(s, bem)
    dt = 1e-4
    rk.step(dt, (1.0, 0.0, 0.0), 1)
    torch.cuda.synchronize()
    u = (X.cpu().numpy().astype(np.float64) - x) / dt
    # potential flow past a sphere of radius 1, U = (1, 0, 0), at the step's midpoint
    xm = x.astype(np.float64) + 0.5 * dt * u
    rr = np.linalg.norm(xm, axis=0)
    cos = xm[0] / rr
    ur = cos * (1 - 1 / rr ** 3)
    ut = -(1 + 0.5 / rr ** 3)
    # u = ur e_r + ut sin(theta) e_theta, with sin(theta) e_theta = (cos e_r - e_x)
    er = xm / rr
    ex = np.array([1.0, 0.0, 0.0])[:, None]
    ref = ur * er + ut * (cos * er - ex)
    err = np.sqrt(((u - ref) ** 2).sum(0).mean())
    assert err <= 2e-2, err


def test_attach_body_rejects_bad_arguments(cuda):
    import ctypes
    s = _sphere(1, 2)
    x, sv, r, _ = _particles(200, 41)
    rk = G.Ralston(_t(x), _t(sv), _t(r), _t(np.ones(x.shape[1], np.float32)))
    arr = s.device_arrays("cuda")
    st = G.influence.surface_struct(arr)
    lib = L.lib()
    wrong = G.BEM(s.npanels * 3)
    assert lib.o3g_rk2_attach_body(rk.h, ctypes.byref(st), 2, 3, wrong.h, 1e-10, 30, 0.0, None) == 1
    right = G.BEM(s.npanels * 2)
    assert lib.o3g_rk2_attach_body(rk.h, ctypes.byref(st), 2, 5, right.h, 1e-10, 30, 0.0, None) == 1
    assert lib.o3g_rk2_attach_body(rk.h, ctypes.byref(st), 4, 3, right.h, 1e-10, 30, 0.0, None) == 1
    assert lib.o3g_rk2_attach_body(rk.h, ctypes.byref(st), 2, 3, right.h, 1e-10, 30, -1.0, None) == 1
    assert lib.o3g_rk2_body_stats(rk.h, None, None, None, None, None) == 9
    L.check(lib.o3g_rk2_attach_body(rk.h, ctypes.byref(st), 2, 3, right.h, 1e-10, 30, 0.0, None), "attach")
    assert lib.o3g_rk2_attach_body(rk.h, ctypes.byref(st), 2, 3, right.h, 1e-10, 30, 0.0, None) == 9


@pytest.mark.parametrize("with_bc", [False, True])
def test_represent_as_particles_bit_exact(cuda, with_bc):
    s = _sphere(3, 2)
    arr = s.device_arrays("cuda")
    rng = np.random.default_rng(17)
    bc1 = rng.normal(size=s.npanels).astype(np.float32) if with_bc else None
    bc2 = rng.normal(size=s.npanels).astype(np.float32) if with_bc else None
    px, ps = G.represent_as_particles(s, 0.0125, bc=(_t(bc1), _t(bc2)) if with_bc else None, arrays=arr)
    po, so = O.represent_as_particles(s.x, s.idx, s.area, s.x1, s.x2, s.norm, 0.0125, s.ts, bc1, bc2)
    assert np.array_equal(px.cpu().numpy(), po) and np.array_equal(ps.cpu().numpy(), so)


def test_shed_particles_after_bem_solve(cuda):
    """Diffusion.h:184-224: solve_bem for the current particles, then one particle per panel
    0.01 h_nu above the surface with the solved panel strength, appended to the last
    collection with core radius vdelta; positions and strengths bit-identical to the
    oracle's represent_as_particles of the solved strengths."""
    x, i = G.generate_ovoid(2, 2.0, 2.0, 2.0)
    surf = G.Surfaces(x, i, nunk=2)
    px, ps, pr = W.shell_particles(2000, seed=31)
    vort = [G.Points(px, ps, pr)]
    bem = G.BEM(surf.npanels * 2)
    h_nu, vdelta = 0.05, 0.02
    nx, ns = G.shed_particles((1.0, 0.0, 0.0), vort, surf, bem, h_nu, vdelta)
    assert vort[0].n == 2000 + surf.npanels
    assert np.array_equal(vort[0].x[:, 2000:], nx) and np.array_equal(vort[0].s[:, 2000:], ns)
    assert np.all(vort[0].r[2000:] == np.float32(vdelta))
    off = float(np.float32(0.01 * float(np.float32(h_nu))))
    ox, os_ = O.represent_as_particles(surf.x, surf.idx, surf.area, surf.x1, surf.x2, surf.norm, off, surf.ts)
    assert np.array_equal(nx.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(ns.view(np.uint32), os_.view(np.uint32))
    assert np.abs(ns).max() > 0
