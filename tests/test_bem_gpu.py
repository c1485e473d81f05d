"""GPU tests of the BEM system through the C-ABI: FP32 LU with partial pivoting (TF32
trailing updates) plus FP64-residual refinement, and GMRES on the unfactored matrix (the
reference's own solver), against an FP64 LU oracle (numpy/LAPACK on the same matrix) and
the potential-flow known answer on a sphere.

Tolerances: refined solutions reach ||b - A x||/||b|| <= 1e-10 (FP64 residual of the FP32
matrix) and agree with the FP64 LU solution of the same matrix to 1e-9 relative (the
matrices here have condition numbers below 1e3)."""
import ctypes

import numpy as np
import pytest

import oracle as O
import omega3d_gb300 as G
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _solve(A, b, tol=1e-10, max_iter=30, method="lu", restart=60):
    n = A.shape[0]
    bem = G.BEM(n)
    bem.set_block(0, 0, np.ascontiguousarray(A.T.astype(np.float32)))   # column-major block
    x, x64 = bem.solve(b.astype(np.float32), tol=tol, max_iter=max_iter, x64=True, method=method, restart=restart)
    return bem, x, x64


@pytest.mark.parametrize("n", [1, 7, 128, 129, 1000, 2500])
def test_lu_refined_solve_matches_fp64_lu(cuda, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    b = rng.normal(size=n)
    bem, x, x64 = _solve(A, b)
    A32 = A.astype(np.float32).astype(np.float64)
    b32 = b.astype(np.float32).astype(np.float64)
    xref = np.linalg.solve(A32, b32)
    assert bem.relres <= 1e-10
    assert np.linalg.norm(b32 - A32 @ x64) / np.linalg.norm(b32) <= 1e-10
    assert np.abs(x64 - xref).max() <= 1e-9 * np.abs(xref).max()
    assert np.abs(x - xref).max() <= 1e-6 * np.abs(xref).max()


def test_pivoting_is_required_and_done(cuda):
    # zero diagonal everywhere: LU without row interchanges fails at the first column
    n = 700
    rng = np.random.default_rng(1)
    P = np.eye(n)[rng.permutation(n)]
    A = P @ (np.eye(n) * 3.0 + rng.normal(size=(n, n)) / np.sqrt(n))
    np.fill_diagonal(A, 0.0)
    b = rng.normal(size=n)
    bem, x, x64 = _solve(A, b)
    A32 = A.astype(np.float32).astype(np.float64)
    assert np.linalg.norm(b.astype(np.float32) - A32 @ x64) / np.linalg.norm(b.astype(np.float32)) <= 1e-10


def test_singular_matrix_is_reported(cuda):
    n = 300
    rng = np.random.default_rng(2)
    A = rng.normal(size=(n, n))
    A[:, 17] = 0.0
    bem = G.BEM(n)
    bem.set_block(0, 0, np.ascontiguousarray(A.T.astype(np.float32)))
    with pytest.raises(G.O3GError) as ei:
        bem.factor()
    assert ei.value.status == 7


def test_solve_before_factor_and_bad_args(cuda):
    lib = L.lib()
    h = ctypes.c_void_p()
    assert lib.o3g_bem_create(0, ctypes.byref(h)) == 1
    L.check(lib.o3g_bem_create(16, ctypes.byref(h)), "create")
    b = np.ones(16, np.float32)
    x = np.zeros(16, np.float32)
    it, rr = ctypes.c_int32(), ctypes.c_double()
    assert lib.o3g_bem_solve(h, b.ctypes.data, x.ctypes.data, None, 0, 1e-10, 5, ctypes.byref(it),
                             ctypes.byref(rr), None) == 9
    blk = np.ones((4, 4), np.float32)
    assert lib.o3g_bem_set_block(h, 14, 4, 0, 4, blk.ctypes.data, 0, None) == 1
    L.check(lib.o3g_bem_destroy(h), "destroy")


@pytest.mark.parametrize("nunk", [2, 3])
def test_sphere_bem_vs_fp64_lu_oracle(cuda, nunk):
    import torch
    x, i = G.generate_ovoid(3, 2.0, 2.0, 2.0)          # unit sphere, 1280 panels
    s = G.Surfaces(x, i, nunk=nunk)
    px, ps, pr = W.shell_particles(4000, seed=31)
    bem = G.BEM(s.npanels * nunk)
    xs = G.solve_bem((1.0, 0.0, 0.0), [G.Points(px, ps, pr)], s, bem)
    assert bem.relres <= 1e-10 and bem.iters <= 10
    # oracle: the same RHS from the oracle's points_affect_panels + finalize + vels_to_rhs,
    # and the GPU-assembled matrix solved by LAPACK in FP64
    pu = O.points_affect_panels(px, ps, s.x, s.idx, s.area, "rm", 1)
    O.finalize_vels(pu, None, (1.0, 0.0, 0.0))
    rhs = O.vels_to_rhs_panels(pu, s.x1, s.x2, s.norm, nunk)
    arr = s.device_arrays("cuda")
    n = s.npanels * nunk
    Ac = torch.empty((n, n), device="cuda")
    G.panels_on_panels_coeff(arr, arr, nunk, True, Ac)
    A = Ac.cpu().numpy().T.astype(np.float64)
    xref = np.linalg.solve(A, rhs.astype(np.float64))
    assert np.abs(xs - xref).max() <= 1e-5 * np.abs(xref).max()


def test_sphere_potential_flow_slip_speed(cuda):
    # inviscid flow past a sphere: the vortex sheet strength equals the slip speed 1.5 U sin(theta)
    x, i = G.generate_ovoid(4, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=2)
    bem = G.BEM(s.npanels * 2)
    G.solve_bem((1.0, 0.0, 0.0), [], s, bem)
    gam = s.ps[0][None, :] * s.x1 + s.ps[1][None, :] * s.x2
    f = i.reshape(-1, 3)
    cen = (x[:, f[:, 0]] + x[:, f[:, 1]] + x[:, f[:, 2]]) / 3
    th = np.arccos(np.clip(cen[0] / np.linalg.norm(cen, axis=0), -1, 1))
    ref = 1.5 * np.sin(th)
    mag = np.linalg.norm(gam, axis=0)
    assert np.sqrt(((mag - ref) ** 2).mean()) / np.sqrt((ref ** 2).mean()) < 5e-3
    # the sheet is tangential and turns the flow around the body: gamma . (n x U) > 0
    assert np.abs((gam * s.norm).sum(0)).max() < 1e-6


def test_panel_vels_to_rhs_matches_oracle(cuda):
    import torch
    x, i = G.generate_ovoid(2, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=3)
    rng = np.random.default_rng(4)
    pu = rng.normal(size=(3, s.npanels)).astype(np.float32)
    fs = (0.3, -1.0, 2.0)
    for nunk in (2, 3):
        pr = pu.copy()
        O.finalize_vels(pr, None, fs)
        ref = O.vels_to_rhs_panels(pr, s.x1, s.x2, s.norm, nunk)
        arr = s.device_arrays("cuda")
        P = torch.from_numpy(pu.copy()).cuda()
        rhs = torch.empty(s.npanels * nunk, device="cuda")
        st = G.influence.surface_struct(arr)
        L.check(L.lib().o3g_panel_vels_to_rhs(s.npanels, nunk, (ctypes.c_double * 3)(*fs),
                                              *[P.data_ptr() + k * s.npanels * 4 for k in range(3)],
                                              ctypes.byref(st), rhs.data_ptr(), None), "rhs")
        torch.cuda.synchronize()
        assert np.array_equal(rhs.cpu().numpy(), ref)
        assert np.array_equal(P.cpu().numpy(), pr)


@pytest.mark.parametrize("n", [1, 7, 129, 1000, 2500])
def test_gmres_matches_fp64_lu(cuda, n):
    rng = np.random.default_rng(100 + n)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    b = rng.normal(size=n)
    bem, x, x64 = _solve(A, b, method="gmres", max_iter=200)
    A32 = A.astype(np.float32).astype(np.float64)
    b32 = b.astype(np.float32).astype(np.float64)
    xref = np.linalg.solve(A32, b32)
    # the residual is checked independently of the library's own FP64-accurate products
    assert bem.relres <= 1e-10
    assert np.linalg.norm(b32 - A32 @ x64) / np.linalg.norm(b32) <= 1e-10
    assert np.abs(x64 - xref).max() <= 1e-9 * np.abs(xref).max()


def test_gmres_restarts_and_reports_non_convergence(cuda):
    n = 600
    rng = np.random.default_rng(5)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 1.2 * np.eye(n)       # slower convergence
    b = rng.normal(size=n)
    bem, x, x64 = _solve(A, b, method="gmres", max_iter=400, restart=8)   # many restarts
    A32 = A.astype(np.float32).astype(np.float64)
    assert np.linalg.norm(b.astype(np.float32) - A32 @ x64) / np.linalg.norm(b.astype(np.float32)) <= 1e-10
    assert bem.iters > 8
    with pytest.raises(G.O3GError) as ei:
        _solve(A, b, method="gmres", max_iter=3)
    assert ei.value.status == 5


@pytest.mark.parametrize("nunk", [2, 3])
def test_sphere_gmres_agrees_with_lu_and_fp64(cuda, nunk):
    import torch
    x, i = G.generate_ovoid(3, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=nunk)
    n = s.npanels * nunk
    arr = s.device_arrays("cuda")
    bem = G.BEM(n)
    bem.assemble(arr, arr, nunk, True)
    rng = np.random.default_rng(nunk)
    b = torch.from_numpy(rng.normal(size=n).astype(np.float32)).cuda()
    xg, xg64 = bem.solve(b, tol=1e-11, max_iter=200, x64=True, method="gmres")
    it_g = bem.iters
    xl, xl64 = bem.solve(b, tol=1e-11, x64=True, method="lu")
    Ac = torch.empty((n, n), device="cuda")
    G.panels_on_panels_coeff(arr, arr, nunk, True, Ac)
    A = Ac.cpu().numpy().T.astype(np.float64)
    xref = np.linalg.solve(A, b.cpu().numpy().astype(np.float64))
    for v in (xg64, xl64):
        assert np.abs(v.cpu().numpy() - xref).max() <= 1e-9 * np.abs(xref).max()
    assert it_g <= 60       # a well-conditioned second-kind system


@pytest.mark.parametrize("method", ["lu", "gmres"])
@pytest.mark.parametrize("nrhs", [1, 2, 3, 8, 11])
def test_many_right_hand_sides_match_fp64_lu(cuda, method, nrhs):
    """o3g_bem_solve_many / o3g_bem_solve_gmres_many: every column against an FP64 LU of the
    same FP32 matrix (1e-9 relative) and to ||b - A x|| / ||b|| <= 1e-10; the columns come out
    as the single-vector solves give them (1e-9 relative); 11 columns run in two groups;
    host and device memory give the same bits."""
    import torch
    n = 1500
    rng = np.random.default_rng(70 + nrhs)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    B = rng.normal(size=(nrhs, n)).astype(np.float32)
    B[0] *= 1e-3                                   # uneven scales converge at different sweeps
    bem = G.BEM(n)
    bem.set_block(0, 0, np.ascontiguousarray(A.T.astype(np.float32)))
    X, X64 = bem.solve_many(B, tol=1e-10, max_iter=300 if method == "gmres" else 30, method=method, x64=True)
    assert (bem.relres_many <= 1e-10).all() and bem.iters_many.shape == (nrhs,)
    A32 = A.astype(np.float32).astype(np.float64)
    Xref = np.linalg.solve(A32, B.astype(np.float64).T).T
    for c in range(nrhs):
        assert np.linalg.norm(B[c] - A32 @ X64[c]) / np.linalg.norm(B[c]) <= 1e-10
        assert np.abs(X64[c] - Xref[c]).max() <= 1e-9 * np.abs(Xref[c]).max()
        x1, x164 = bem.solve(B[c], tol=1e-10, max_iter=300 if method == "gmres" else 30, method=method, x64=True)
        assert np.abs(X64[c] - x164).max() <= 1e-9 * np.abs(x164).max()
    Xg, Xg64 = bem.solve_many(torch.from_numpy(B).cuda(), tol=1e-10, max_iter=300 if method == "gmres" else 30,
                              method=method, x64=True)
    torch.cuda.synchronize()
    assert np.array_equal(Xg64.cpu().numpy(), X64)


def test_many_right_hand_sides_empty_and_zero_columns(cuda):
    n = 300
    rng = np.random.default_rng(80)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    bem = G.BEM(n)
    bem.set_block(0, 0, np.ascontiguousarray(A.T.astype(np.float32)))
    for method in ("lu", "gmres"):
        X = bem.solve_many(np.zeros((0, n), np.float32), method=method)
        assert X.shape == (0, n)
        B = np.stack([np.zeros(n, np.float32), rng.normal(size=n).astype(np.float32)])
        X = bem.solve_many(B, tol=1e-10, max_iter=300, method=method)
        assert not X[0].any() and bem.relres_many[1] <= 1e-10


@pytest.mark.parametrize("nunk", [2, 3])
def test_gmres_block_preconditioner(cuda, nunk):
    """GMRES right-preconditioned by the inverses of the panels' diagonal blocks
    (o3g_bem_set_unknowns_per_panel, set by BEM.assemble on a surface's own block): the
    same solution as FP64 LU of the same matrix (1e-9 of max |x|) with the unpreconditioned
    iteration as well, for one and for several right-hand sides, and fewer iterations with
    3 unknowns per panel (vortex and source sheets)."""
    import torch
    x, i = G.generate_ovoid(3, 2.0, 2.0, 2.0)
    s = G.Surfaces(x, i, nunk=nunk)
    n = s.npanels * nunk
    arr = s.device_arrays("cuda")
    bem = G.BEM(n)
    bem.assemble(arr, arr, nunk, True)
    Ac = torch.empty((n, n), device="cuda")
    G.panels_on_panels_coeff(arr, arr, nunk, True, Ac)
    A = Ac.cpu().numpy().T.astype(np.float64)
    rng = np.random.default_rng(10 + nunk)
    B = rng.normal(size=(3, n)).astype(np.float32)
    xref = np.linalg.solve(A, B.astype(np.float64).T).T
    scale = np.abs(xref).max(axis=1)
    b = torch.from_numpy(B[0]).cuda()
    _, xp64 = bem.solve(b, tol=1e-11, max_iter=300, x64=True, method="gmres")
    it_pre = bem.iters
    assert np.abs(xp64.cpu().numpy() - xref[0]).max() <= 1e-9 * scale[0]
    bem.set_unknowns_per_panel(1)
    _, x064 = bem.solve(b, tol=1e-11, max_iter=300, x64=True, method="gmres")
    it_none = bem.iters
    assert np.abs(x064.cpu().numpy() - xref[0]).max() <= 1e-9 * scale[0]
    if nunk == 3:
        assert it_pre < it_none
    else:
        assert it_pre <= it_none
    bem.set_unknowns_per_panel(nunk)
    X, X64 = bem.solve_many(torch.from_numpy(B).cuda(), tol=1e-11, max_iter=300, x64=True, method="gmres")
    assert (bem.relres_many <= 1e-11).all()
    for c in range(3):
        assert np.abs(X64[c].cpu().numpy() - xref[c]).max() <= 1e-9 * scale[c]
    # block size 1..3 dividing n
    with pytest.raises(G.O3GError):
        bem.set_unknowns_per_panel(4)
    if n % 3 != 0:
        with pytest.raises(G.O3GError):
            bem.set_unknowns_per_panel(3)
