"""GPU tests of the bounded device-side waits.

The BEM panel factorisation and triangular solves synchronise their blocks with grid
barriers, and the particle split's dependency chain waits for flags that earlier particles
publish.  Every such wait has a limit; one that runs out sets an error word, the others
then return at once, the kernels end and the call returns O3G_ERR_TIMEOUT with the device
still usable.  o3g_debug_wait_test(1) gives those waits a condition nothing fulfils (a
barrier count one above the number of blocks, a flag nothing sets) and a limit of about a
millisecond.  Each test checks that the call gives up with O3G_ERR_TIMEOUT, switches the
test off, and checks that the next calls succeed with correct results.  No wait is left
unbounded and nothing traps."""
import ctypes

import numpy as np
import pytest

import oracle as O
import omega3d_gb300 as G
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TIMEOUT = 6


def _wait_test(on):
    assert L.lib().o3g_debug_wait_test(1 if on else 0) == 0


def test_bem_barriers_run_out_and_the_next_calls_succeed(cuda):
    lib = L.lib()
    n = 1000
    rng = np.random.default_rng(60)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    b = rng.normal(size=n).astype(np.float32)
    bem = G.BEM(n)
    bem.set_block(0, 0, np.ascontiguousarray(A.T.astype(np.float32)))
    _wait_test(True)
    try:
        st = lib.o3g_bem_factor(bem.h, None)
    finally:
        _wait_test(False)
    assert st == TIMEOUT, lib.o3g_last_error().decode()
    assert "timed out" in lib.o3g_last_error().decode()
    # the factorisation runs again and the solve converges
    bem.factor()
    x, x64 = bem.solve(b, tol=1e-10, max_iter=30, x64=True)
    A32 = A.astype(np.float32).astype(np.float64)
    xref = np.linalg.solve(A32, b.astype(np.float64))
    assert bem.relres <= 1e-10 and np.abs(x64 - xref).max() <= 1e-9 * np.abs(xref).max()
    # the triangular solves' barriers
    xo = np.zeros(n, np.float32)
    it, rr = ctypes.c_int32(), ctypes.c_double()
    _wait_test(True)
    try:
        st = lib.o3g_bem_solve(bem.h, b.ctypes.data, xo.ctypes.data, None, L.MEM_HOST, 1e-10, 5, ctypes.byref(it),
                               ctypes.byref(rr), None)
    finally:
        _wait_test(False)
    assert st == TIMEOUT, lib.o3g_last_error().decode()
    x2, x264 = bem.solve(b, tol=1e-10, max_iter=30, x64=True)
    assert bem.relres <= 1e-10 and np.array_equal(x264, x64)


def test_split_waits_run_out_and_leave_the_particles_unchanged(cuda):
    lib = L.lib()
    x, s, r, e = W.lattice_particles(k=16, seed=61, elong_scale=0.1)
    e[:] = np.float32(1.5)                       # every particle splits: long dependency chains
    n = x.shape[1]
    want = O.split_elongated(x, s, r, e, 0, 1.5, 1.2)
    cap = 2 * n

    def arrays():
        X = torch.full((3, cap), float("nan"), device="cuda")
        S = torch.full((3, cap), float("nan"), device="cuda")
        R = torch.full((cap,), float("nan"), device="cuda")
        E = torch.full((cap,), float("nan"), device="cuda")
        X[:, :n], S[:, :n], R[:n], E[:n] = (torch.from_numpy(a).cuda() for a in (x, s, r, e))
        return X, S, R, E

    def call(X, S, R, E):
        m = ctypes.c_int32()
        rows = lambda t: [t.data_ptr() + k * cap * 4 for k in range(3)]  # noqa: E731
        st = lib.o3g_split_elongated(n, cap, *rows(X), R.data_ptr(), E.data_ptr(), *rows(S), 0, 1.5, 1.2,
                                     ctypes.byref(m), None)
        torch.cuda.synchronize()
        return st, m.value

    X, S, R, E = arrays()
    before = [t.cpu().numpy().copy() for t in (X, S, R, E)]
    _wait_test(True)
    try:
        st, _ = call(X, S, R, E)
    finally:
        _wait_test(False)
    assert st == TIMEOUT, lib.o3g_last_error().decode()
    for t, b0 in zip((X, S, R, E), before):
        assert np.array_equal(t.cpu().numpy().view(np.uint32), b0.view(np.uint32))
    # the next split succeeds, bit for bit the oracle's
    st, m = call(X, S, R, E)
    assert st == 0 and m == n == want[4]
    for t, w in zip((X, S, R, E), want[:4]):
        assert np.array_equal(t.cpu().numpy().view(np.uint32), w.view(np.uint32))
