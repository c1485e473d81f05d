"""Parity at the full sizes of the measured configurations, through properties that do not
need a CPU sum over all pairs:

* the 262,144-particle precision cloud (Gaussian core): exact linearity in the strengths,
  superposition, and the compensated and plain paths against the FP64 path on the same GPU
  at 2,048 seeded targets (all sources);
* the 40,960-unknown sphere system (20,480 panels, 100,000 particles): GMRES and the LU path
  both reach 1e-10 and agree with each other;
* the 1,048,576-particle wake (RM core, compensated): sums against the FP64 path at 1,024
  seeded targets;
* the 64 seeded blob systems in one batched launch: 8 systems against the FP64 path.

Bounds (stated per test): compensated L-infinity (max |du| / max |u| over the sample)
<= 1e-6, per-target relative <= 1e-5 (2e-5 on the strongly cancelling blobs); plain
L-infinity <= 2e-5."""
import numpy as np
import pytest

import omega3d_gb300 as G
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import linf_err, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _sums(x, s, r, core, prec):
    p = G.Points(_t(x), _t(s), _t(r))
    G.points_affect_points(p, p, G.ResultsType(), G.ExecEnv(core, prec))
    torch.cuda.synchronize()
    return p.u.cpu().numpy(), p.ug.cpu().numpy()


def _fp64_at(x, s, r, sub, core):
    tq = G.Points(_t(x[:, sub].astype(np.float64)), None, _t(r[sub].astype(np.float64)))
    G.points_affect_points(G.Points(_t(x.astype(np.float64)), _t(s.astype(np.float64)), _t(r.astype(np.float64))),
                           tq, G.ResultsType(), G.ExecEnv(core, "fp64"))
    torch.cuda.synchronize()
    return tq.u.cpu().numpy(), tq.ug.cpu().numpy()


def test_precision_cloud_full_size(cuda):
    n = 262144
    x, s, r = W.gaussian_cloud(n, seed=2)
    sub = np.sort(np.random.default_rng(17).choice(n, 2048, replace=False))
    u64, g64 = _fp64_at(x, s, r, sub, "gauss")
    uc, gc = _sums(x, s, r, "gauss", "compensated")
    assert linf_err(uc[:, sub], u64) <= 1e-6 and linf_err(gc[:, sub], g64) <= 1e-6
    assert rel_err(uc[:, sub], u64)[0] <= 1e-5 and rel_err(gc[:, sub], g64)[0] <= 1e-5
    up, gp = _sums(x, s, r, "gauss", "plain")
    assert linf_err(up[:, sub], u64) <= 2e-5 and linf_err(gp[:, sub], g64) <= 2e-5
    # doubling every strength doubles every sum exactly (every product and two-sum scales by 2)
    u2, g2 = _sums(x, 2 * s, r, "gauss", "compensated")
    assert np.array_equal(u2, 2 * uc) and np.array_equal(g2, 2 * gc)
    # superposition of two halves of the strength field
    sa = (s * np.float32(0.25)).astype(np.float32)
    sb = (s - sa).astype(np.float32)
    ua, ga = _sums(x, sa, r, "gauss", "compensated")
    ub, gb = _sums(x, sb, r, "gauss", "compensated")
    assert linf_err(ua + ub, uc) <= 1e-6 and linf_err(ga + gb, gc) <= 1e-6


def test_sphere_bem_full_size(cuda):
    """20,480 panels, 2 unknowns per panel: RHS from 100,000 shell particles and (1,0,0);
    GMRES (the reference's method) and the refined LU both to 1e-10, agreeing to 1e-8."""
    x, i = G.generate_ovoid(5, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=2)
    arr = s.device_arrays("cuda")
    px, ps, pr = W.shell_particles(100000, seed=3)
    src = G.Points(_t(px), _t(ps), _t(pr))
    n = s.npanels * 2
    pu = torch.zeros(3, s.npanels, device="cuda")
    G.points_affect_panels(src, s, arrays=arr, pu=pu)
    rhs = torch.empty(n, device="cuda")
    st = G.influence.surface_struct(arr)
    fsd = (G.influence.ctypes.c_double * 3)(1.0, 0.0, 0.0)
    G.lib().o3g_panel_vels_to_rhs(s.npanels, 2, fsd, *G.influence._rows(pu, 3), G.influence.ctypes.byref(st),
                                  rhs.data_ptr(), None)
    bem = G.BEM(n)
    bem.assemble(arr, arr, 2, True)
    xg = bem.solve(rhs, tol=1e-10, max_iter=300, method="gmres")
    assert bem.relres <= 1e-10 and bem.iters < 60
    bem.factor()
    xl = bem.solve(rhs, tol=1e-10, max_iter=30)
    assert bem.relres <= 1e-10
    torch.cuda.synchronize()
    assert float(((xg - xl).abs().max() / xl.abs().max()).item()) <= 1e-8


def test_wake_particles_full_size(cuda):
    n = 1048576
    x, s, r = W.wake_particles(n, seed=5)
    sub = np.sort(np.random.default_rng(19).choice(n, 1024, replace=False))
    u64, g64 = _fp64_at(x, s, r, sub, "rm")
    uc, gc = _sums(x, s, r, "rm", "compensated")
    assert linf_err(uc[:, sub], u64) <= 1e-6 and linf_err(gc[:, sub], g64) <= 1e-6
    assert rel_err(uc[:, sub], u64)[0] <= 1e-5


def test_batch_64_systems_full_size(cuda):
    """The 64 seeded blob systems (1,024 to 65,536 particles, 4,096 field points each) in one
    compensated Gaussian launch; 8 of them checked against the FP64 path for that system
    alone, particles and field points.  These blobs cancel strongly at some targets, where
    FP32 pair terms alone give up to 6.5e-6 per target, so the per-target bound is 2e-5."""
    systems = W.batch_systems(64, seed=4)
    devs = []
    for x, s, r, f in systems:
        n, nf = x.shape[1], f.shape[1]
        devs.append(G.BatchSystem(_t(x), _t(s), _t(r), torch.zeros((3, n), device="cuda"),
                                  torch.zeros((9, n), device="cuda"), _t(f), torch.zeros((3, nf), device="cuda"),
                                  torch.zeros((9, nf), device="cuda")))
    G.Batch(devs, G.ExecEnv("gauss", "compensated"), grads=True).run()
    torch.cuda.synchronize()
    for k in range(0, 64, 8):
        x, s, r, f = systems[k]
        src = G.Points(_t(x.astype(np.float64)), _t(s.astype(np.float64)), _t(r.astype(np.float64)))
        tp = G.Points(_t(x.astype(np.float64)), None, _t(r.astype(np.float64)))
        tf = G.Points(_t(f.astype(np.float64)), None, None, inert=True)
        for tq in (tp, tf):
            G.points_affect_points(src, tq, G.ResultsType(), G.ExecEnv("gauss", "fp64"))
        torch.cuda.synchronize()
        d = devs[k]
        for got_u, got_g, ref in ((d.u, d.ug, tp), (d.fu, d.fug, tf)):
            u, g = got_u.cpu().numpy(), got_g.cpu().numpy()
            u64, g64 = ref.u.cpu().numpy(), ref.ug.cpu().numpy()
            assert linf_err(u, u64) <= 1e-6 and linf_err(g, g64) <= 1e-6
            assert rel_err(u, u64)[0] <= 2e-5 and rel_err(g, g64)[0] <= 2e-5
