"""GPU parity tests of points_affect_points through the C-ABI (libo3dgpu.so).

Tolerances (per-target relative error, metrics.rel_err, floor 1e-6 of the max):
  * PLAIN vs the reference's FP32 pair arithmetic with double accumulators (the
    reference's non-Vc build, Simulation.h:44-46; oracle prec 1): max <= 1e-5, the
    FP32-summation-reordering tolerance of the drop-in path.
  * PLAIN vs the golden vectors of the reference's Vc-semantics build (prec 0): max <= 1e-5.
  * EXP core: PLAIN evaluates 1 - exp(-x) in float exactly as the reference does
    (CoreFunc.h:127-128, :175-177), so it is held to the same 1e-5; that float form loses
    ~eps/x near the core, so against the FP64 oracle PLAIN may deviate as far as the
    reference's own float build does (x1.5, floor 1e-5).  COMPENSATED and FP64 use expm1.
  * COMPENSATED vs the FP64 oracle: L-infinity (metrics.linf_err) <= 1e-6 and
    per-target max <= 1e-5 (FP32 rounding of single pair terms bounds the latter).
  * FP64 vs the FP64 oracle / golden: max <= 1e-11.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle as O
from omega3d_gb300 import ExecEnv, Points, ResultsType, points_affect_points
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import linf_err, rel_err

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CORES = ["rm", "wl", "exp", "gauss", "v2"]


def _dev(a, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a if dtype is None else a.astype(dtype)))
    return t.cuda()


def gpu_eval(sx, ss, sr, tx, tr, grads=True, core="rm", prec="plain", on_device=True, dtype=np.float32,
             u0=None, g0=None):
    import torch
    cv = (lambda a: _dev(a, dtype)) if on_device else (lambda a: np.ascontiguousarray(a.astype(dtype)))
    src = Points(cv(sx), cv(ss), cv(sr))
    targ = Points(cv(tx), None, None if tr is None else cv(tr), inert=tr is None, grads=grads,
                  u=None if u0 is None else cv(u0), ug=None if g0 is None else cv(g0))
    points_affect_points(src, targ, ResultsType("velandgrad" if grads else "velonly"), ExecEnv(core, prec))
    if on_device:
        torch.cuda.synchronize()
        u = targ.u.cpu().numpy()
        g = targ.ug.cpu().numpy() if grads else None
    else:
        u, g = targ.u, (targ.ug if grads else None)
    return u, g


@pytest.mark.parametrize("core", CORES)
@pytest.mark.parametrize("kind", ["particles", "fieldpoints"])
def test_plain_matches_reference_fp32_semantics(cuda, core, kind):
    x, s, r = W.gaussian_cloud(3000, seed=101, pos_std=0.25)
    tx, _, tr = W.gaussian_cloud(2100, seed=102, pos_std=0.25)
    tr = tr if kind == "particles" else None
    tol = 1e-5
    uo, go = O.points_affect_points(x, r, s, tx, tr, True, core, 1)
    u, g = gpu_eval(x, s, r, tx, tr, True, core, "plain")
    eu, eg = rel_err(u, uo), rel_err(g, go)
    assert eu[0] <= tol and eg[0] <= tol, (eu, eg)
    if core == "exp":
        u64, g64 = O.points_affect_points(x, r, s, tx, tr, True, core, 2)
        bu = max(1e-5, 1.5 * rel_err(uo, u64)[0])
        bg = max(1e-5, 1.5 * rel_err(go, g64)[0])
        assert rel_err(u, u64)[0] <= bu and rel_err(g, g64)[0] <= bg
    uo, _ = O.points_affect_points(x, r, s, tx, tr, False, core, 1)
    u, _ = gpu_eval(x, s, r, tx, tr, False, core, "plain")
    assert rel_err(u, uo)[0] <= tol


@pytest.mark.parametrize("core", CORES)
def test_golden_vectors(cuda, core):
    d = np.load(os.path.join(GOLD, "ptpt_%s.npz" % core))
    tol = 1e-5
    for tr, tag in ((d["tr"], "pg"), (None, "fg")):
        u, g = gpu_eval(d["sx"], d["ss"], d["sr"], d["tx"], tr, True, core, "plain")
        assert rel_err(u, d[tag + "_u_p0"])[0] <= tol
        assert rel_err(g, d[tag + "_g_p0"])[0] <= tol
        u, g = gpu_eval(d["sx"], d["ss"], d["sr"], d["tx"], tr, True, core, "fp64", dtype=np.float64)
        assert rel_err(u, d[tag + "_u_p2"])[0] <= 1e-11
        assert rel_err(g, d[tag + "_g_p2"])[0] <= 1e-11
    u, _ = gpu_eval(d["sx"], d["ss"], d["sr"], d["tx"], d["tr"], False, core, "plain")
    assert rel_err(u, d["pv_u_p0"])[0] <= tol


@pytest.mark.parametrize("core", CORES)
def test_compensated_and_fp64_vs_fp64_oracle(cuda, core):
    x, s, r = W.gaussian_cloud(6000, seed=103, pos_std=0.3)
    tx = x[:, :1500].copy()
    tr = r[:1500].copy()
    uo, go = O.points_affect_points(x, r, s, tx, tr, True, core, 2)
    u, g = gpu_eval(x, s, r, tx, tr, True, core, "compensated")
    eu, eg = rel_err(u, uo), rel_err(g, go)
    lu, lg = linf_err(u, uo), linf_err(g, go)
    print("compensated", core, eu, eg, lu, lg)
    assert lu <= 1e-6 and lg <= 1e-6, (lu, lg)
    assert eu[0] <= 1e-5 and eg[0] <= 1e-5, (eu, eg)
    # the float-input FP64 mode rounds only the final sums to float
    u, g = gpu_eval(x, s, r, tx, tr, True, core, "fp64")
    assert rel_err(u, uo)[0] <= 2e-7 and rel_err(g, go)[0] <= 2e-7
    # the double entry point
    u, g = gpu_eval(x, s, r, tx, tr, True, core, "fp64", dtype=np.float64)
    assert rel_err(u, uo)[0] <= 1e-11 and rel_err(g, go)[0] <= 1e-11


def test_host_and_device_memory_give_identical_bits(cuda):
    x, s, r = W.gaussian_cloud(1000, seed=104)
    tx, _, tr = W.gaussian_cloud(777, seed=105)
    for prec in ("plain", "compensated"):
        a = gpu_eval(x, s, r, tx, tr, True, "rm", prec, on_device=True)
        b = gpu_eval(x, s, r, tx, tr, True, "rm", prec, on_device=False)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_accumulates_into_existing_values(cuda):
    x, s, r = W.gaussian_cloud(500, seed=106)
    tx, _, tr = W.gaussian_cloud(300, seed=107)
    u0 = np.random.default_rng(0).normal(size=(3, 300)).astype(np.float32)
    g0 = np.random.default_rng(1).normal(size=(9, 300)).astype(np.float32)
    a = gpu_eval(x, s, r, tx, tr, True, "wl", "plain")
    b = gpu_eval(x, s, r, tx, tr, True, "wl", "plain", u0=u0, g0=g0)
    assert np.allclose(b[0], a[0] + u0, rtol=1e-6, atol=1e-6 * np.abs(a[0]).max())
    assert np.allclose(b[1], a[1] + g0, rtol=1e-6, atol=1e-6 * np.abs(a[1]).max())


@pytest.mark.parametrize("ns,nt", [(1, 1), (1, 300), (129, 1), (127, 129), (255, 257), (4097, 33)])
def test_ragged_sizes(cuda, ns, nt):
    x, s, r = W.gaussian_cloud(ns, seed=108 + ns)
    tx, _, tr = W.gaussian_cloud(nt, seed=109 + nt)
    for core in ("rm", "gauss"):
        uo, go = O.points_affect_points(x, r, s, tx, tr, True, core, 1)
        u, g = gpu_eval(x, s, r, tx, tr, True, core, "plain")
        assert rel_err(u, uo)[0] <= 1e-5 and rel_err(g, go)[0] <= 1e-5


def test_empty_inputs_are_noops(cuda):
    x, s, r = W.gaussian_cloud(10, seed=110)
    e = np.zeros((3, 0), np.float32)
    u, g = gpu_eval(e, e, np.zeros(0, np.float32), x, r, True, "rm", "plain")
    assert np.all(u == 0) and np.all(g == 0)
    u, g = gpu_eval(x, s, r, e, np.zeros(0, np.float32), True, "rm", "plain")
    assert u.shape == (3, 0)


def test_self_interaction_same_arrays(cuda):
    import torch
    x, s, r = W.vortex_ring(2048, seed=111)
    X, S, R = _dev(x), _dev(s), _dev(r)
    p = Points(X, S, R)
    points_affect_points(p, p, ResultsType(), ExecEnv("rm", "plain"))
    q = Points(X.clone(), None, R.clone())
    points_affect_points(Points(X, S, R), q, ResultsType(), ExecEnv("rm", "plain"))
    torch.cuda.synchronize()
    assert torch.equal(p.u, q.u) and torch.equal(p.ug, q.ug)


def test_linearity_in_strength_at_full_ring_size(cuda):
    # scaling every strength by 2 scales every sum by exactly 2 (all products scale by a power of 2)
    import torch
    x, s, r = W.vortex_ring(16384)
    a = gpu_eval(x, s, r, x, r, True, "rm", "plain")
    b = gpu_eval(x, 2 * s, r, x, r, True, "rm", "plain")
    assert np.array_equal(2 * a[0], b[0]) and np.array_equal(2 * a[1], b[1])
    # and agrees with the reference semantics on a subset of targets
    idx = np.arange(0, 16384, 64)
    uo, go = O.points_affect_points(x, r, s, x[:, idx], r[idx], True, "rm", 1)
    assert rel_err(a[0][:, idx], uo)[0] <= 1e-5 and rel_err(a[1][:, idx], go)[0] <= 1e-5


def test_invalid_arguments_report_status(cuda):
    lib = L.lib()
    st = lib.o3g_points_affect_points(9, 0, 1, 1, *([None] * 7), 1, *([None] * 4), *([None] * 3), None, None)
    assert st == 1
    assert lib.o3g_last_error().decode()


def _per_pair_err(test, ref):
    """|test_i - ref_i| / |ref_i| per target (no floor: every target here sees one source);
    targets whose reference is exactly zero must be exactly zero."""
    t = np.asarray(test, np.float64)
    r = np.asarray(ref, np.float64)
    nr = np.sqrt((r * r).sum(axis=0))
    d = np.sqrt(((t - r) ** 2).sum(axis=0))
    zero = nr == 0
    assert not d[zero].any()
    return np.where(zero, 0.0, d / np.where(zero, 1.0, nr))


@pytest.mark.parametrize("core", CORES)
def test_branch_edges_vs_reference_build(cuda, core):
    """One source, targets where the cores switch form (tests/golden/branch_edges.npz, from
    the reference's own kernels; the Gaussian core from the oracle): d^3/sigma^3 around 0.001
    and 16 (the exponential core's branches, CoreFunc.h:119-177) and around q = 48 (the
    Gaussian core's far switch), d = 0, and extreme separations, for particle targets, field
    points and velocity-only targets, in every precision.

    Per-pair tolerances (no summation is involved):
      * PLAIN vs the reference's float build: 5e-6, the hardware reciprocal square root
        (<= 2 ulp) through r^-3 and r^-5.  EXP between the branches adds what the float
        form 1 - exp(-x) makes of the exp results: CUDA's expf and the host's libm may
        differ by up to ~3 ulp, which 1 - e amplifies by e/(1 - e), so 4 ulp(1) e/(1 - e)
        more (2.4e-4 at x = 0.001, 5e-7 at x = 1).
      * COMPENSATED vs the reference's FP64 build: 2e-6.  At the exponential core's exact
        switch points (d^3/sigma^3 = 0.001 and 16 to the rounding of the inputs) a float and
        a double evaluation of the same pair may land on either side, as the reference's own
        float and double builds do, so there the bound is the jump, 6e-4.
      * FP64 (double entry point) vs FP64 build: 1e-11.
    """
    d = np.load(os.path.join(GOLD, "branch_edges.npz"))
    rel = d["rel"]
    e = np.exp(-rel)
    mid = (rel >= 1e-3 * 0.999) & (rel <= 16.0 * 1.001)
    tol_p = np.full(rel.size, 5e-6)
    tol_c = np.full(rel.size, 2e-6)
    if core == "exp":
        tol_p = tol_p + np.where(mid, 4 * 2.0 ** -24 * e / np.maximum(-np.expm1(-rel), 1e-30), 0.0)
        tol_c[np.isclose(rel, 1e-3, rtol=1e-9) | np.isclose(rel, 16.0, rtol=1e-9)] = 6e-4
    for tag, tx, tr in (("pg", d["tx_p"], d["tr"]), ("fg", d["tx_f"], None)):
        u, g = gpu_eval(d["sx"], d["ss"], d["sr"], tx, tr, True, core, "plain")
        eu = _per_pair_err(u, d["%s_%s_u_p0" % (core, tag)])
        eg = _per_pair_err(g, d["%s_%s_g_p0" % (core, tag)])
        assert (eu <= tol_p).all() and (eg <= tol_p).all(), (tag, eu.max(), eg.max(), rel[np.argmax(eg / tol_p)])
        u, g = gpu_eval(d["sx"], d["ss"], d["sr"], tx, tr, True, core, "compensated")
        eu = _per_pair_err(u, d["%s_%s_u_p2" % (core, tag)])
        eg = _per_pair_err(g, d["%s_%s_g_p2" % (core, tag)])
        assert (eu <= tol_c).all() and (eg <= tol_c).all(), (tag, eu.max(), eg.max())
        u, g = gpu_eval(d["sx"], d["ss"], d["sr"], tx, tr, True, core, "fp64", dtype=np.float64)
        assert _per_pair_err(u, d["%s_%s_u_p2" % (core, tag)]).max() <= 1e-11
        assert _per_pair_err(g, d["%s_%s_g_p2" % (core, tag)]).max() <= 1e-11
    u, _ = gpu_eval(d["sx"], d["ss"], d["sr"], d["tx_p"], d["tr"], False, core, "plain")
    assert (_per_pair_err(u, d["%s_pv_u_p0" % core]) <= tol_p).all()
    u, _ = gpu_eval(d["sx"], d["ss"], d["sr"], d["tx_p"], d["tr"], False, core, "compensated")
    assert (_per_pair_err(u, d["%s_pv_u_p2" % core]) <= tol_c).all()


@pytest.mark.parametrize("method", [(1, 0), (0, 0), (3, 1)])
def test_reference_external_hook(cuda, method):
    """external_vel_solver_f_ / _d_ with the reference's exact prototypes (Influence.h:33-48):
    by-pointer counts, host arrays, targets summed as points (no target radius), results
    added to what the arrays hold, the reference's flop count returned.  Float: against the
    oracle's float pair arithmetic (prec 1) at 1e-5 (COMPENSATED: FP64 oracle, 1e-5);
    double: against the FP64 oracle at 1e-11.  A second call adds the same sums again
    (L-infinity 1e-6 of twice the first)."""
    lib = L.lib()
    core, prec = method
    name = [k for k, v in L.CORES.items() if v == core][0]
    assert lib.o3g_external_set_method(core, prec) == 0
    try:
        x, s, r = W.gaussian_cloud(1500, seed=120, pos_std=0.25)
        tx, _, _ = W.gaussian_cloud(700, seed=121, pos_std=0.25)
        for dt, ref_prec, tol, fn in ((np.float32, 1 if prec == 0 else 2, 1e-5, lib.external_vel_solver_f_),
                                      (np.float64, 2, 1e-11, lib.external_vel_solver_d_)):
            X, S, R, T = (np.ascontiguousarray(a.astype(dt)) for a in (x, s, r, tx))
            u = np.zeros((3, 700), dt)
            g = np.zeros((9, 700), dt)
            ns, nt = ctypes.c_int(1500), ctypes.c_int(700)
            row = lambda a, k: a[k].ctypes.data  # noqa: E731
            args = [ctypes.byref(ns), row(X, 0), row(X, 1), row(X, 2), row(S, 0), row(S, 1), row(S, 2),
                    R.ctypes.data, ctypes.byref(nt), row(T, 0), row(T, 1), row(T, 2),
                    row(u, 0), row(u, 1), row(u, 2)] + [row(g, k) for k in range(9)]
            flops = fn(*args)
            assert flops == pytest.approx(700 * (12.0 + lib.o3g_flops_per_pair(core, 1, 0) * 1500), rel=1e-6)
            uo, go = O.points_affect_points(x, r, s, tx, None, True, name, ref_prec)
            assert rel_err(u, uo)[0] <= tol and rel_err(g, go)[0] <= tol
            u1, g1 = u.copy(), g.copy()
            assert fn(*args) > 0
            assert linf_err(u, 2 * u1) <= 1e-6 and linf_err(g, 2 * g1) <= 1e-6
    finally:
        lib.o3g_external_set_method(-1, -1)


def test_exponential_core_exp_is_nearly_correctly_rounded(cuda):
    """The plain exponential core's float exp (o3g_exp_probe) over the range it serves,
    -16 < x < -0.001 (log-uniform), and over [-20, 0]: at most 1 ulp from the correctly
    rounded float, and different from it for no more than 1e-4 of the arguments (the host
    library's float exp, glibc's, is within 0.502 ulp: this keeps 1 - exp(-x) on the
    reference's values)."""
    import torch
    rng = np.random.default_rng(31)
    x = np.concatenate([-np.exp(rng.uniform(np.log(1e-3), np.log(16.02), 1 << 20)),
                        rng.uniform(-20.0, 0.0, 1 << 18)]).astype(np.float32)
    X = torch.from_numpy(x).cuda()
    Y = torch.empty_like(X)
    assert L.lib().o3g_exp_probe(x.size, X.data_ptr(), Y.data_ptr(), None) == 0
    torch.cuda.synchronize()
    y = Y.cpu().numpy()
    cr = np.exp(x.astype(np.float64)).astype(np.float32)
    ulp = np.abs(y.view(np.int32).astype(np.int64) - cr.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1
    assert np.count_nonzero(ulp) <= 1e-4 * x.size
