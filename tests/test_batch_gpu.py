"""GPU tests of the batched persistent pair sums (o3g_batch_*) and the batched Ralston
stepper (o3g_batch_rk2_create) through the C-ABI.

Every system of a batch must receive what points_affect_points gives for that system
alone: its particles are the sources, its particles (thick-cored) and its field points
(inert) the targets.  Tolerances as for the single-system path (per-target relative
error, metrics.rel_err):
  * PLAIN vs the oracle with FP32 pair arithmetic and double accumulation (prec 1):
    L-infinity <= 1e-5, and per target <= max(1e-5, 4 d), d = how far the reference's own
    FP32-accumulation semantics (prec 0) are from prec 1 on the same system.  The blobs
    here cancel strongly at some targets, where d itself reaches 1.6e-5: FP32 sums in other
    orders land 0.6-1.5e-5 away (emulated), and the hardware rsqrt (<= 2 ulp, approximate
    like the reference's Vc::rsqrt) adds about as much again.  The EXP core's PLAIN form
    is the reference's float 1 - exp(-x), held to the same bound;
  * COMPENSATED vs the FP64 oracle: L-infinity <= 1e-6, and per target <= max(1e-5, 3 d1),
    d1 = the per-target error of FP32 pair terms summed exactly (oracle prec 1) on the same
    system: compensated sums remove the summation error, not the rounding of the FP32 pair
    terms, which reaches 6.5e-6 (1e-5 for EXP gradients) at the strongly cancelling targets
    of these blobs.
"""
import ctypes
import inspect
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
import omega3d_gb300 as G
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import linf_err, rel_err

pytestmark = pytest.mark.gpu
CORES = ["rm", "wl", "exp", "gauss", "v2"]
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _systems(sizes, fields, seed):
    rng = np.random.default_rng(seed)
    out = []
    for n, nf in zip(sizes, fields):
        sb = rng.uniform(0.1, 0.4)
        x = rng.normal(0.0, sb, (3, n)).astype(np.float32)
        s = (rng.normal(0.0, 1.0, (3, n)) * 1e-3).astype(np.float32)
        r = rng.uniform(0.01, 0.05, n).astype(np.float32)
        f = rng.uniform(-2 * sb, 2 * sb, (3, nf)).astype(np.float32)
        out.append((x, s, r, f))
    return out


def _make(systems, grads=True, u0=None):
    import torch
    devs = []
    for i, (x, s, r, f) in enumerate(systems):
        n, nf = x.shape[1], f.shape[1]
        u = _t(u0[i][0]) if u0 is not None else torch.zeros((3, n), device="cuda")
        ug = (_t(u0[i][1]) if u0 is not None else torch.zeros((9, n), device="cuda")) if grads else None
        fu = torch.zeros((3, nf), device="cuda") if nf else None
        fug = torch.zeros((9, nf), device="cuda") if (nf and grads) else None
        devs.append(G.BatchSystem(_t(x), _t(s), _t(r), u, ug, _t(f) if nf else None, fu, fug))
    return devs


def _results(devs, grads=True):
    import torch
    torch.cuda.synchronize()
    out = []
    for d in devs:
        out.append((d.u.cpu().numpy(), d.ug.cpu().numpy() if grads else None,
                    d.fu.cpu().numpy() if d.fu is not None else None,
                    d.fug.cpu().numpy() if (d.fug is not None and grads) else None))
    return out


def _run(systems, core, prec, grads=True, config=None):
    devs = _make(systems, grads)
    b = G.Batch(devs, G.ExecEnv(core, prec), grads=grads)
    if config is not None:
        b.set_config(*config)
    b.run()
    return _results(devs, grads), b


SIZES = [1, 127, 128, 129, 700, 2000, 0, 3000]
FIELDS = [0, 5, 300, 0, 129, 1000, 50, 0]


@pytest.mark.parametrize("core", CORES)
def test_batch_plain_matches_oracle_per_system(cuda, core):
    systems = _systems(SIZES, FIELDS, seed=400)
    tol = 1e-5
    for grads in (True, False):
        res, _ = _run(systems, core, "plain", grads)
        for (x, s, r, f), (u, g, fu, fg) in zip(systems, res):
            if x.shape[1] == 0:
                if fu is not None:
                    assert not fu.any()
                continue
            for tx, tr, a, b in ((x, r, u, g), (f, None, fu, fg)):
                if tx.shape[1] == 0:
                    continue
                uo, go = O.points_affect_points(x, r, s, tx, tr, grads, core, 1)
                u0, g0 = O.points_affect_points(x, r, s, tx, tr, grads, core, 0)
                assert linf_err(a, uo) <= tol and rel_err(a, uo)[0] <= max(tol, 4 * rel_err(u0, uo)[0])
                if grads:
                    assert linf_err(b, go) <= tol and rel_err(b, go)[0] <= max(tol, 4 * rel_err(g0, go)[0])


@pytest.mark.parametrize("core", ["rm", "gauss", "exp"])
def test_batch_compensated_vs_fp64_oracle(cuda, core):
    systems = _systems([1500, 4000, 2500, 333], [700, 0, 4096, 64], seed=401)
    res, _ = _run(systems, core, "compensated")
    for (x, s, r, f), (u, g, fu, fg) in zip(systems, res):
        for tx, tr, a, b in ((x, r, u, g), (f, None, fu, fg)):
            if tx.shape[1] == 0:
                continue
            uo, go = O.points_affect_points(x, r, s, tx, tr, True, core, 2)
            u1, g1 = O.points_affect_points(x, r, s, tx, tr, True, core, 1)
            assert linf_err(a, uo) <= 1e-6 and linf_err(b, go) <= 1e-6
            assert rel_err(a, uo)[0] <= max(1e-5, 3 * rel_err(u1, uo)[0])
            assert rel_err(b, go)[0] <= max(1e-5, 3 * rel_err(g1, go)[0])


def test_every_configuration_agrees_and_repeats_bit_for_bit(cuda):
    # 4096-particle systems: small chunks make split 16 cut every target block
    systems = _systems([4096, 4096, 1000, 4096], [512, 0, 4096, 100], seed=402)
    ref = None
    for prec, tpts in (("plain", (1, 2, 4)), ("compensated", (1, 2))):
        ref = None
        for tpt in tpts:
            for split in (0, 4, 16):
                for bps in (0, 1):
                    res, b = _run(systems, "gauss", prec, True, (tpt, bps, split))
                    cfg = b.config()
                    assert cfg["tpt"] == tpt and cfg["split"] == split
                    if split == 16 and bps == 0:
                        assert cfg["chunk"] == 8      # the split path (slabs + last arriver) ran
                    again, _ = _run(systems, "gauss", prec, True, (tpt, bps, split))
                    for a, c in zip(res, again):
                        for p, q in zip(a, c):
                            assert (p is None and q is None) or np.array_equal(p, q)
                    if ref is None:
                        ref = res
                        continue
                    for a, c in zip(res, ref):
                        for p, q in zip(a, c):
                            if p is None:
                                continue
                            # summation order differs between configurations: compare the sums'
                            # accuracy (L-infinity); per-target bounds are checked against the oracle
                            assert linf_err(p, q) <= (5e-7 if prec == "compensated" else 5e-6)


def test_batch_accumulates(cuda):
    systems = _systems([300, 900], [0, 0], seed=403)
    rng = np.random.default_rng(5)
    u0 = [(rng.normal(size=(3, x.shape[1])).astype(np.float32), rng.normal(size=(9, x.shape[1])).astype(np.float32))
          for x, _, _, _ in systems]
    devs = _make(systems, True, u0)
    G.Batch(devs, G.ExecEnv("wl", "plain")).run()
    got = _results(devs)
    base, _ = _run(systems, "wl", "plain")
    for (u, g, _, _), (ub, gb, _, _), (a, c) in zip(got, base, u0):
        assert np.allclose(u, ub + a, rtol=1e-6, atol=1e-6 * np.abs(ub).max())
        assert np.allclose(g, gb + c, rtol=1e-6, atol=1e-6 * np.abs(gb).max())


def test_one_shot_entry_point_equals_handle(cuda):
    import torch
    systems = _systems([640, 1300], [256, 10], seed=404)
    res, b = _run(systems, "rm", "compensated")
    devs = _make(systems)
    arr = (L.System * len(devs))(*[d.struct(True) for d in devs])
    L.check(L.lib().o3g_batch_velgrad(0, 1, 1, len(devs), arr, torch.cuda.current_stream().cuda_stream),
            "o3g_batch_velgrad")
    for a, c in zip(res, _results(devs)):
        for p, q in zip(a, c):
            assert (p is None and q is None) or np.array_equal(p, q)


def test_tuned_configuration_is_cached_per_shape(cuda, tmp_path):
    path = str(tmp_path / "tune.txt")
    old = os.environ.get("O3G_TUNE_CACHE")
    os.environ["O3G_TUNE_CACHE"] = path
    try:
        systems = _systems([2222, 1111, 3333], [77, 0, 512], seed=405)
        devs = _make(systems)
        b = G.Batch(devs, G.ExecEnv("gauss", "plain"))
        assert b.config()["tuned"] == 0
        b.run()
        cfg = b.config()
        assert cfg["tuned"] == 1
        rows = [l.split() for l in open(path).read().split("\n") if l.strip()]
        assert any(int(w[1]) == cfg["tpt"] and int(w[3]) == cfg["split"] for w in rows)
        # same shape in this process: configured at creation
        b2 = G.Batch(_make(systems), G.ExecEnv("gauss", "plain"))
        c2 = b2.config()
        assert c2["tuned"] == 1 and c2["tpt"] == cfg["tpt"] and c2["split"] == cfg["split"]
        # and in a fresh process, from the file
        code = ("import json, numpy as np, torch, omega3d_gb300 as G\n" + inspect.getsource(_t) +
                inspect.getsource(_systems) + inspect.getsource(_make) +
                "b = G.Batch(_make(_systems([2222, 1111, 3333], [77, 0, 512], seed=405)), G.ExecEnv('gauss', 'plain'))\n"
                "print(json.dumps(b.config()))\n")
        env = dict(os.environ, O3G_TUNE_CACHE=path, PYTHONPATH=ROOT)
        out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True,
                             timeout=300)
        assert out.returncode == 0, out.stderr
        c3 = json.loads(out.stdout.strip().split("\n")[-1])
        assert c3["tuned"] == 1 and c3["tpt"] == cfg["tpt"] and c3["split"] == cfg["split"]
        # a different shape is not configured
        b4 = G.Batch(_make(_systems([2222, 1111, 3334], [77, 0, 512], seed=405)), G.ExecEnv("gauss", "plain"))
        assert b4.config()["tuned"] == 0
    finally:
        if old is None:
            os.environ.pop("O3G_TUNE_CACHE", None)
        else:
            os.environ["O3G_TUNE_CACHE"] = old


def test_bad_arguments_are_rejected(cuda):
    lib = L.lib()
    systems = _systems([100], [10], seed=406)
    devs = _make(systems)
    arr = (L.System * 1)(devs[0].struct(True))
    h = ctypes.c_void_p()
    assert lib.o3g_batch_create(0, 2, 1, 1, arr, ctypes.byref(h)) == 1          # FP64 not batched
    assert lib.o3g_batch_create(7, 0, 1, 1, arr, ctypes.byref(h)) == 1          # unknown core
    assert lib.o3g_batch_create(0, 0, 1, 0, arr, ctypes.byref(h)) == 1          # no systems
    bad = (L.System * 1)(devs[0].struct(True))
    bad[0].ug[4] = None
    assert lib.o3g_batch_create(0, 0, 1, 1, bad, ctypes.byref(h)) == 1          # gradient array missing
    bad[0].np = -1
    assert lib.o3g_batch_create(0, 0, 0, 1, bad, ctypes.byref(h)) == 1          # negative count
    L.check(lib.o3g_batch_create(0, 1, 1, 1, arr, ctypes.byref(h)), "create")
    assert lib.o3g_batch_set_config(h, 4, 0, 4) == 1                            # tpt 4: not compiled for comp+grads
    assert lib.o3g_batch_set_config(h, 1, 0, 5) == 1                            # split not offered
    L.check(lib.o3g_batch_destroy(h), "destroy")


def _concat(systems):
    x = np.concatenate([s[0] for s in systems], axis=1)
    s = np.concatenate([s[1] for s in systems], axis=1)
    r = np.concatenate([s[2] for s in systems])
    f = np.concatenate([s[3] for s in systems], axis=1)
    return x, s, r, f


def test_batch_ralston_matches_single_system_steppers(cuda):
    import torch
    systems = _systems([1500, 600, 2500], [300, 0, 1000], seed=407)
    x, s, r, f = _concat(systems)
    X, S, R, E, F = _t(x), _t(s), _t(r), _t(np.ones(x.shape[1], np.float32)), _t(f)
    rk = G.BatchRalston([q[0].shape[1] for q in systems], [q[3].shape[1] for q in systems], X, S, R, E, F,
                        G.ExecEnv("rm", "plain"))
    rk.step(0.01, (0.1, 0.0, 0.0), 3)
    torch.cuda.synchronize()
    P = Fo = 0
    for (xi, si, ri, fi) in systems:
        n, nf = xi.shape[1], fi.shape[1]
        Xi, Si, Ri, Ei = _t(xi), _t(si), _t(ri), _t(np.ones(n, np.float32))
        Fi = _t(fi) if nf else None
        G.Ralston(Xi, Si, Ri, Ei, fieldpts=Fi, env=G.ExecEnv("rm", "plain")).step(0.01, (0.1, 0.0, 0.0), 3)
        torch.cuda.synchronize()
        assert rel_err(X[:, P:P + n].cpu().numpy() - xi, Xi.cpu().numpy() - xi)[0] <= 1e-4
        # the stretching term s . grad(u) cancels at some particles: compare the strength
        # changes against the largest one (the gradient sums differ by summation order only)
        assert linf_err(S[:, P:P + n].cpu().numpy() - si, Si.cpu().numpy() - si) <= 1e-4
        assert np.abs(E[P:P + n].cpu().numpy() - Ei.cpu().numpy()).max() <= 1e-5
        if nf:
            assert rel_err(F[:, Fo:Fo + nf].cpu().numpy() - fi, Fi.cpu().numpy() - fi)[0] <= 1e-4
        P += n
        Fo += nf


def test_batch_ralston_graph_replay_equals_direct_steps(cuda):
    import torch
    systems = _systems([900, 2048, 130], [64, 512, 0], seed=408)
    x, s, r, f = _concat(systems)
    outs = []
    for use_graph in (True, False):
        X, S, R, E, F = _t(x), _t(s), _t(r), _t(np.ones(x.shape[1], np.float32)), _t(f)
        rk = G.BatchRalston([q[0].shape[1] for q in systems], [q[3].shape[1] for q in systems], X, S, R, E, F,
                            G.ExecEnv("gauss", "compensated"), use_graph=use_graph)
        rk.step(0.01, (0.0, 0.0, 0.0), 4)
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in (X, S, E, F)])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert not np.array_equal(outs[0][0], x)
