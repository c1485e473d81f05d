"""Particle split and merge on the GPU (o3g_split_elongated / o3g_merge_close_particles,
replacing split_elongated<float>, Split.h:44-270, and merge_close_particles<float>,
Merge.h:45-218): bit-identical to the oracle restatement (pinned to the reference's own
Split.h / Merge.h) and to the golden fixture generated from them."""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "splitmerge.npz")


def _g():
    import omega3d_gb300 as G
    return G


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    assert a.shape == b.shape
    bad = np.nonzero(a.view(np.uint32) != b.view(np.uint32))
    assert bad[0].size == 0, "%d of %d values differ, first at %s: %r vs %r" % (
        bad[0].size, a.size, [int(v[0]) for v in bad], a[tuple(v[0] for v in bad)], b[tuple(v[0] for v in bad)])


def _split_gpu(x, s, r, e, core, overlap=1.5, threshold=1.2):
    G = _g()
    xs, ss, rs, es, m = G.split_elongated(_dev(x), _dev(s), _dev(r), _dev(e), core, overlap, threshold)
    return xs.cpu().numpy(), ss.cpu().numpy(), rs.cpu().numpy(), es.cpu().numpy(), m


def _merge_gpu(x, s, r, overlap=1.5, threshold=0.2, adapt=False):
    G = _g()
    xm, sm, rm, k = G.merge_close_particles(_dev(x), _dev(s), _dev(r), overlap, threshold, adapt)
    return xm.cpu().numpy(), sm.cpu().numpy(), rm.cpu().numpy(), k


@pytest.mark.parametrize("core", [0, 1])
def test_split_golden(core):
    d = np.load(GOLDEN)
    got = _split_gpu(d["x_in"], d["s_in"], d["r_in"], d["e_in"], ["gaussian", "compactg"][core])
    for k, v in zip("xsre", got[:4]):
        _bits_equal(v, d["split%d_%s" % (core, k)])


@pytest.mark.parametrize("name,thr,adapt", [("merge_vrm", 0.2, False), ("merge_core", 0.02, False),
                                            ("merge_amr", 0.2, True)])
def test_merge_golden(name, thr, adapt):
    d = np.load(GOLDEN)
    got = _merge_gpu(d["x_in"], d["s_in"], d["r_in"], 1.5, thr, adapt)
    for k, v in zip("xsr", got[:3]):
        _bits_equal(v, d["%s_%s" % (name, k)])


@pytest.mark.parametrize("core", [0, 1])
def test_split_tied_lattice(core):
    """Unjittered lattice (neighbours at exactly equal distance).  The kernel and the oracle
    both visit ties in increasing index: bit-identical.  Against the reference's own output,
    whose tie order follows its kd-tree: count, positions, radii and elongations
    bit-identical, strengths within 1e-7 of the largest strength magnitude."""
    d = np.load(os.path.join(os.path.dirname(GOLDEN), "splitmerge_tied.npz"))
    x, s, r, e = d["x_in"], d["s_in"], d["r_in"], d["e_in"]
    got = _split_gpu(x, s, r, e, ["gaussian", "compactg"][core])
    want = O.split_elongated(x, s, r, e, core, 1.5, 1.2)
    assert got[4] == want[4] > 0
    for a, b in zip(got[:4], want[:4]):
        _bits_equal(a, b)
    for k in (0, 2, 3):
        _bits_equal(got[k], d["split%d_%s" % (core, "xsre"[k])])
    ref_s = d["split%d_s" % core]
    assert np.abs(got[1].astype(np.float64) - ref_s).max() <= 1e-7 * np.abs(ref_s).max()


@pytest.mark.parametrize("name,thr", [("merge_vrm", 0.2), ("merge_core", 0.02)])
def test_merge_duplicated_particles(name, thr):
    """Lattice particles plus exact copies of a fifth of them.  The kernel and the oracle
    take equal-distance partners in increasing index: bit-identical.  The reference takes
    them in its kd-tree order.  It removes the same number and keeps the same total
    strength, but at threshold 0.2 it keeps other members of some coincident pairs."""
    d = np.load(os.path.join(os.path.dirname(GOLDEN), "splitmerge_tied.npz"))
    xd, sd, rd = d["xd_in"], d["sd_in"], d["rd_in"]
    got = _merge_gpu(xd, sd, rd, 1.5, thr, False)
    want = O.merge_close_particles(xd, sd, rd, 1.5, thr, False)
    assert got[3] == want[3] > 0
    for a, b in zip(got[:3], want[:3]):
        _bits_equal(a, b)
    ref_s = d[name + "_s"]
    assert got[3] == xd.shape[1] - ref_s.shape[1]
    assert np.allclose(got[1].astype(np.float64).sum(1), ref_s.astype(np.float64).sum(1), rtol=0, atol=1e-7)


@pytest.mark.parametrize("k,scale,core", [(40, 0.12, 0), (40, 0.05, 1), (100, 0.12, 0)])
def test_split_vs_oracle(k, scale, core):
    """64,000 and 1,000,000 particles; with the 0.12 tail 19 % split and the dependency
    chain through lower-index split neighbours is hundreds deep."""
    from omega3d_gb300 import workloads as W
    x, s, r, e = W.lattice_particles(k=k, seed=21, elong_scale=scale)
    want = O.split_elongated(x, s, r, e, core, 1.5, 1.2)
    got = _split_gpu(x, s, r, e, ["gaussian", "compactg"][core])
    assert got[4] == want[4] > 0
    for a, b in zip(got[:4], want[:4]):
        _bits_equal(a, b)


@pytest.mark.parametrize("overlap", [1.0, 2.0])
def test_split_merge_mixed_radii_vs_oracle(overlap):
    """Unequal core radii (lattice radius times U[0.7, 1.3]) and other overlaps and
    thresholds: the cell size follows the largest search radius, every match test and
    weight the pair's own radii."""
    from omega3d_gb300 import workloads as W
    x, s, r, e = W.lattice_particles(k=16, seed=34, overlap=overlap, elong_scale=0.2)
    r = (r * np.random.default_rng(35).uniform(0.7, 1.3, r.size)).astype(np.float32)
    for core in (0, 1):
        want = O.split_elongated(x, s, r, e, core, overlap, 1.05)
        got = _split_gpu(x, s, r, e, ["gaussian", "compactg"][core], overlap, 1.05)
        assert got[4] == want[4] > 0
        for a, b in zip(got[:4], want[:4]):
            _bits_equal(a, b)
    for thr, adapt in ((0.05, False), (0.5, True)):
        want = O.merge_close_particles(x, s, r, overlap, thr, adapt)
        got = _merge_gpu(x, s, r, overlap, thr, adapt)
        assert got[3] == want[3] > 0
        for a, b in zip(got[:3], want[:3]):
            _bits_equal(a, b)


def test_split_every_particle_elongated():
    """Every particle split: the longest dependency chain the operator can have here."""
    from omega3d_gb300 import workloads as W
    x, s, r, e = W.lattice_particles(k=24, seed=22, elong_scale=0.1)
    e[:] = np.float32(1.5)
    want = O.split_elongated(x, s, r, e, 0, 1.5, 1.2)
    got = _split_gpu(x, s, r, e, "gaussian")
    assert got[4] == x.shape[1]
    for a, b in zip(got[:4], want[:4]):
        _bits_equal(a, b)


@pytest.mark.parametrize("k,thr,adapt", [(40, 0.2, False), (40, 0.02, False), (40, 0.2, True), (100, 0.2, False)])
def test_merge_vs_oracle(k, thr, adapt):
    from omega3d_gb300 import workloads as W
    x, s, r, _ = W.lattice_particles(k=k, seed=23)
    want = O.merge_close_particles(x, s, r, 1.5, thr, adapt)
    got = _merge_gpu(x, s, r, 1.5, thr, adapt)
    assert got[3] == want[3] > 0
    for a, b in zip(got[:3], want[:3]):
        _bits_equal(a, b)


def test_merge_clusters_and_duplicates():
    """Dense clusters (groups of many particles, long greedy sequences) and exact duplicates
    (ties in distance, visited in index order by both the oracle and the kernel)."""
    rng = np.random.default_rng(24)
    c = rng.uniform(-1, 1, (3, 200))
    x = np.repeat(c, 20, axis=1) + rng.normal(scale=0.002, size=(3, 4000))
    x[:, 1::7] = x[:, 0::7][:, :x[:, 1::7].shape[1]]
    x = x.astype(np.float32)
    s = (rng.normal(size=(3, 4000)) * 1e-3).astype(np.float32)
    r = rng.uniform(0.01, 0.03, 4000).astype(np.float32)
    for adapt in (False, True):
        want = O.merge_close_particles(x, s, r, 1.5, 0.2, adapt)
        got = _merge_gpu(x, s, r, 1.5, 0.2, adapt)
        assert got[3] == want[3] > 1000
        for a, b in zip(got[:3], want[:3]):
            _bits_equal(a, b)


def test_split_merge_edges():
    G = _g()
    from omega3d_gb300 import workloads as W
    x, s, r, e = W.lattice_particles(k=10, seed=25)
    # nothing elongated: unchanged, same tensors back
    e1 = np.ones_like(e)
    tx, ts, tr, te = _dev(x), _dev(s), _dev(r), _dev(e1)
    out = G.split_elongated(tx, ts, tr, te)
    assert out[4] == 0 and out[0] is tx
    # capacity too small: the C-ABI reports the count and changes nothing
    import ctypes
    te = _dev(e)
    ns = ctypes.c_int32()
    from omega3d_gb300 import _lib as L
    rows = lambda a, k: [a.data_ptr() + i * a.shape[1] * 4 for i in range(k)]   # noqa: E731
    st = L.lib().o3g_split_elongated(x.shape[1], x.shape[1], *rows(tx, 3), tr.data_ptr(), te.data_ptr(),
                                     *rows(ts, 3), 0, 1.5, 1.2, ctypes.byref(ns), None)
    assert st == 10 and ns.value == int(np.count_nonzero(e > np.float32(1.2)))
    torch.cuda.synchronize()
    _bits_equal(tx.cpu().numpy(), x)
    _bits_equal(te.cpu().numpy(), e)
    # bad arguments
    assert L.lib().o3g_split_elongated(-1, 0, *([None] * 8), 0, 1.5, 1.2, ctypes.byref(ns), None) == 1
    assert L.lib().o3g_split_elongated(5, 5, *([None] * 8), 7, 1.5, 1.2, ctypes.byref(ns), None) == 1
    assert L.lib().o3g_merge_close_particles(5, *([None] * 7), 1.5, 0.2, 0, ctypes.byref(ns), None) == 1
    # empty sets
    z3 = torch.zeros((3, 0), device="cuda")
    z1 = torch.zeros(0, device="cuda")
    assert G.split_elongated(z3, z3.clone(), z1, z1.clone())[4] == 0
    assert G.merge_close_particles(z3, z3.clone(), z1)[3] == 0
    # far apart: nothing merges
    xf = (np.arange(3 * 50, dtype=np.float32).reshape(3, 50) * 10).astype(np.float32)
    got = _merge_gpu(xf, s[:, :50].copy(), r[:50].copy())
    assert got[3] == 0
    _bits_equal(got[0], xf)


def test_too_many_matches_refused():
    """48,000 coincident particles: every one matches every other, 2.3e9 matches in all,
    more than the int offsets of the match lists can index.  Both operators refuse with
    INVALID_ARG before writing anything, and the arrays come back unchanged."""
    G = _g()
    from omega3d_gb300._lib import O3GError
    n = 48000
    x = np.full((3, n), 0.25, np.float32)
    s = np.zeros((3, n), np.float32)
    s[0] = 1e-4
    r = np.full(n, 0.015, np.float32)
    e = np.full(n, 2.0, np.float32)
    tx, ts, tr, te = _dev(x), _dev(s), _dev(r), _dev(e)
    for call in (lambda: G.split_elongated(tx, ts, tr, te), lambda: G.merge_close_particles(tx, ts, tr)):
        with pytest.raises(O3GError, match="2\\^31") as ex:
            call()
        assert ex.value.status == 1
    torch.cuda.synchronize()
    for a, b in ((tx, x), (ts, s), (tr, r), (te, e)):
        _bits_equal(a.cpu().numpy(), b)
    # the library stays usable
    xs, ss, rs, es, m = _split_gpu(*_small_lattice(), "gaussian")
    assert m > 0


def _small_lattice():
    from omega3d_gb300 import workloads as W
    return W.lattice_particles(k=8, seed=26)


def test_split_merge_deterministic():
    from omega3d_gb300 import workloads as W
    x, s, r, e = W.lattice_particles(k=40, seed=26)
    a = _split_gpu(x, s, r, e, "gaussian")
    b = _split_gpu(x, s, r, e, "gaussian")
    for u, v in zip(a[:4], b[:4]):
        _bits_equal(u, v)
    a = _merge_gpu(x, s, r)
    b = _merge_gpu(x, s, r)
    for u, v in zip(a[:3], b[:3]):
        _bits_equal(u, v)
