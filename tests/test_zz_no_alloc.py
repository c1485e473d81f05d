"""GPU test of o3g_points_affect_points_noalloc, the entry point for callers that may not
allocate device memory (programs that hand all device memory to their own pool, real-time
loops, plugin hosts that forbid allocation after start-up).  Its scratch lives in a fixed
array inside the library, so the test calls it twice in a row -- the second call finds the
first call's leftovers in that array -- and checks both results against the allocating
entry point o3g_points_affect_points, for every core, and against the oracle.  The two
entry points split the sources differently, so PLAIN compares two FP32 summation orders:
L-infinity <= 1e-5 and per target <= 3e-5 (orders land up to 1.5e-5 apart where a sum
cancels strongly, as in the batch tests); against the oracle's float pair arithmetic with
double sums, per target <= 3e-5.  COMPENSATED: L-infinity <= 1e-6 and per target <= 1e-5,
against the allocating entry point and against the oracle's FP64 sums.  The library's
allocation counter (o3g_alloc_count) must not move across the no-allocation calls, and a
fresh process whose first library call is this entry point makes no allocation at all.

This file is named to be collected last, so a run that stops at the first failure has
run every other test before it; it also passes on its own in a fresh process.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import linf_err, rel_err

pytestmark = pytest.mark.gpu


def _rows(t):
    n = t.shape[1]
    return [t.data_ptr() + k * n * 4 for k in range(t.shape[0])]


def _call(fn, core, prec, X, S, R, TX, TR, U, G, stream, with_mem):
    sx, ss, tx, tu = _rows(X), _rows(S), _rows(TX), _rows(U)
    tug = (ctypes.c_void_p * 9)(*_rows(G)) if G is not None else None
    tr = TR.data_ptr() if TR is not None else None
    head = [core, prec, L.MEM_DEVICE] if with_mem else [core, prec]
    return fn(*head, X.shape[1], *sx, R.data_ptr(), *ss, TX.shape[1], *tx, tr, *tu, tug, stream)


def _allocs(lib):
    n = ctypes.c_uint64()
    assert lib.o3g_alloc_count(ctypes.byref(n)) == 0
    return n.value


@pytest.mark.parametrize("core", ["rm", "wl", "exp", "gauss", "v2"])
@pytest.mark.parametrize("prec", ["plain", "compensated"])
@pytest.mark.parametrize("case", ["self", "fieldpoints"])
def test_noalloc_matches_allocating_entry_point_twice(cuda, core, prec, case):
    import torch
    lib = L.lib()
    x, s, r = W.gaussian_cloud(5000, seed=201)
    X, S, R = (torch.from_numpy(a).cuda() for a in (x, s, r))
    if case == "self":
        TX, TR = X, R
    else:
        tx, _, _ = W.gaussian_cloud(3001, seed=202)
        TX, TR = torch.from_numpy(tx).cuda(), None
    nt = TX.shape[1]
    stream = torch.cuda.current_stream().cuda_stream
    c, p = L.CORES[core], L.PRECS[prec]

    U0 = torch.zeros(3, nt, device="cuda")
    G0 = torch.zeros(9, nt, device="cuda")
    L.check(_call(lib.o3g_points_affect_points, c, p, X, S, R, TX, TR, U0, G0, stream, True),
            "o3g_points_affect_points")
    torch.cuda.synchronize()
    u0, g0 = U0.cpu().numpy(), G0.cpu().numpy()

    tx_np = TX.cpu().numpy()
    tr_np = None if TR is None else TR.cpu().numpy()
    uo, go = O.points_affect_points(x, r, s, tx_np, tr_np, True, core, 1 if prec == "plain" else 2)
    for _ in range(2):
        U = torch.zeros(3, nt, device="cuda")
        G = torch.zeros(9, nt, device="cuda")
        torch.cuda.synchronize()
        before = _allocs(lib)
        L.check(_call(lib.o3g_points_affect_points_noalloc, c, p, X, S, R, TX, TR, U, G, stream, False),
                "o3g_points_affect_points_noalloc")
        torch.cuda.synchronize()
        assert _allocs(lib) == before
        u, g = U.cpu().numpy(), G.cpu().numpy()
        tol = 3e-5 if prec == "plain" else 1e-5
        assert rel_err(u, uo)[0] <= tol and rel_err(g, go)[0] <= tol
        if prec == "plain":
            # the two entry points split the sources differently: two FP32 summation orders,
            # which land up to 1.5e-5 apart per target where the sum cancels strongly
            assert linf_err(u, u0) <= 1e-5 and linf_err(g, g0) <= 1e-5
            assert rel_err(u, u0)[0] <= 3e-5 and rel_err(g, g0)[0] <= 3e-5
        else:
            assert linf_err(u, u0) <= 1e-6 and linf_err(g, g0) <= 1e-6
            assert rel_err(u, u0)[0] <= 1e-5 and rel_err(g, g0)[0] <= 1e-5


def test_noalloc_velocity_only_and_rejections(cuda):
    import torch
    lib = L.lib()
    x, s, r = W.gaussian_cloud(2000, seed=203)
    X, S, R = (torch.from_numpy(a).cuda() for a in (x, s, r))
    stream = torch.cuda.current_stream().cuda_stream
    U0 = torch.zeros(3, 2000, device="cuda")
    U = torch.zeros(3, 2000, device="cuda")
    L.check(_call(lib.o3g_points_affect_points, 1, 0, X, S, R, X, R, U0, None, stream, True), "allocating")
    L.check(_call(lib.o3g_points_affect_points_noalloc, 1, 0, X, S, R, X, R, U, None, stream, False), "noalloc")
    torch.cuda.synchronize()
    assert rel_err(U.cpu().numpy(), U0.cpu().numpy())[0] <= 1e-5
    # FP64 is not offered without allocation
    assert _call(lib.o3g_points_affect_points_noalloc, 0, 2, X, S, R, X, R, U, None, stream, False) == 1
    # a problem whose packed tiles exceed the fixed array is refused before any work is
    # queued (the buffers are real and large enough, so nothing could be read out of range)
    n = 2_200_000
    BX = torch.zeros(3, n, device="cuda")
    BR = torch.ones(n, device="cuda")
    BU = torch.zeros(3, n, device="cuda")
    st = _call(lib.o3g_points_affect_points_noalloc, 0, 0, BX, BX, BR, BX, BR, BU, None, stream, False)
    assert st == 1
    assert "scratch" in lib.o3g_last_error().decode()


_FRESH = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W
lib = L.lib()
x, s, r = W.gaussian_cloud(3000, seed=204)
X, S, R = (torch.from_numpy(a).cuda() for a in (x, s, r))
rows = lambda t: [t.data_ptr() + k * t.shape[1] * 4 for k in range(t.shape[0])]
out = []
for _ in range(2):
    U = torch.zeros(3, 3000, device="cuda")
    G = torch.zeros(9, 3000, device="cuda")
    tug = (ctypes.c_void_p * 9)(*rows(G))
    st = lib.o3g_points_affect_points_noalloc(3, 1, 3000, *rows(X), R.data_ptr(), *rows(S), 3000, *rows(X),
                                              R.data_ptr(), *rows(U), tug, None)
    assert st == 0, lib.o3g_last_error()
    torch.cuda.synchronize()
    out.append((U.cpu().numpy(), G.cpu().numpy()))
n = ctypes.c_uint64()
assert lib.o3g_alloc_count(ctypes.byref(n)) == 0
assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
print("allocs", n.value)
"""


def test_noalloc_first_call_in_a_fresh_process_allocates_nothing(cuda):
    """A process whose first library call is the no-allocation entry point: two calls, the
    library's allocation counter stays at zero, and the second call (which finds the first
    one's leftovers in the shared array) gives the same bits."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "allocs 0" in r.stdout
