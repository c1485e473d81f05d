"""CPU tests of the batched path's work-item plan (o3g_batch_plan, host only): every
(target block, source tile) pair of every system is covered by exactly one item, items
run longest first, split target blocks own distinct partial-sum slabs, and no item is
longer than the chunk the plan promises."""
import ctypes

import numpy as np
import pytest

from omega3d_gb300 import _lib as L

KB = 128   # threads per block == sources per tile


def plan(np_, nf, tpt, grid, split):
    lib = L.lib()
    n = len(np_)
    a = (ctypes.c_int32 * n)(*np_)
    b = (ctypes.c_int32 * n)(*nf)
    ni, nt, ch = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    ns = ctypes.c_int64()
    L.check(lib.o3g_batch_plan(n, a, b, tpt, grid, split, ctypes.byref(ni), ctypes.byref(nt), ctypes.byref(ch),
                               ctypes.byref(ns), None, None), "o3g_batch_plan")
    items = np.zeros((max(ni.value, 1), 4), np.int32)
    tbs = np.zeros((max(nt.value, 1), 4), np.int32)
    L.check(lib.o3g_batch_plan(n, a, b, tpt, grid, split, None, None, None, None, items.ctypes.data,
                               tbs.ctypes.data), "o3g_batch_plan")
    return items[:ni.value], tbs[:nt.value], ch.value, ns.value


def check_plan(np_, nf, tpt, grid, split):
    items, tbs, chunk, nslabs = plan(np_, nf, tpt, grid, split)
    TB = KB * tpt
    tiles = [(n + KB - 1) // KB for n in np_]
    t0 = np.concatenate([[0], np.cumsum(tiles)])
    # target blocks: one per TB targets of every system with sources, slots back to back
    slot = 0
    k = 0
    for i, (n, f) in enumerate(zip(np_, nf)):
        nb = (n + f + TB - 1) // TB if n > 0 else 0
        for b in range(nb):
            assert tbs[k, 0] == i and tbs[k, 1] == slot
            slot += TB
            k += 1
    assert k == len(tbs)
    # coverage: each target block's tiles exactly once, split indices 0..nsplit-1
    cover = {}
    for tb, a, e, q in items:
        assert a < e and e - a <= chunk
        sysi = tbs[tb, 0]
        assert t0[sysi] <= a and e <= t0[sysi + 1]
        cover.setdefault(tb, []).append((q, a, e))
    slabs = set()
    for tb in range(len(tbs)):
        parts = sorted(cover[tb])
        assert [p[0] for p in parts] == list(range(tbs[tb, 3]))
        sysi = tbs[tb, 0]
        edges = [t0[sysi]] + [p[2] for p in parts]
        assert [p[1] for p in parts] == edges[:-1] and edges[-1] == t0[sysi + 1]
        if tbs[tb, 3] > 1:
            for q in range(tbs[tb, 3]):
                assert tbs[tb, 2] + q not in slabs
                slabs.add(tbs[tb, 2] + q)
        else:
            assert tbs[tb, 2] == -1
    assert len(slabs) == nslabs and (not slabs or max(slabs) == nslabs - 1)
    # longest first
    lens = items[:, 2] - items[:, 1]
    assert np.all(np.diff(lens) <= 0)
    return items, tbs, chunk


@pytest.mark.parametrize("tpt", [1, 2, 4])
@pytest.mark.parametrize("split", [0, 4, 16])
def test_plan_covers_every_pair_once(built_lib, tpt, split):
    rng = np.random.default_rng(4)
    np_ = [int(round(np.exp(rng.uniform(np.log(1024), np.log(65536))))) for _ in range(64)]
    nf = [4096] * 64
    items, tbs, chunk = check_plan(np_, nf, tpt, 608, split)
    if split == 0:
        assert len(items) == len(tbs)
    else:
        units = sum(((n + f + KB * tpt - 1) // (KB * tpt)) * ((n + KB - 1) // KB) for n, f in zip(np_, nf))
        assert chunk == max(8, -(-units // (608 * split)))


def test_plan_ragged_and_empty_systems(built_lib):
    check_plan([0, 1, 127, 128, 129, 0, 5000], [10, 0, 3, 0, 1000, 0, 0], 2, 152, 16)
    items, tbs, _ = check_plan([0], [100], 1, 152, 4)
    assert len(items) == 0 and len(tbs) == 0


def test_plan_rejects_bad_arguments(built_lib):
    lib = L.lib()
    a = (ctypes.c_int32 * 1)(10)
    b = (ctypes.c_int32 * 1)(0)
    assert lib.o3g_batch_plan(1, a, b, 3, 152, 4, None, None, None, None, None, None) == 1
    assert lib.o3g_batch_plan(0, a, b, 1, 152, 4, None, None, None, None, None, None) == 1
    assert lib.o3g_batch_plan(1, a, b, 1, 0, 4, None, None, None, None, None, None) == 1
    neg = (ctypes.c_int32 * 1)(-1)
    assert lib.o3g_batch_plan(1, neg, b, 1, 152, 4, None, None, None, None, None, None) == 1
