"""TEST INFRASTRUCTURE ONLY.

numpy front end of the C++ oracle (oracle/o3d_oracle.cpp) and of the reference-kernel
libraries built by oracle/build_ref.sh into oracle/_ref/.  Arrays are component-major
SoA exactly like the reference's std::array<Vector<S>,3> (x[3, n]); gradients are
[9, n] in the reference order (Kernels.h:184-192).

prec 0: S=A=float (reference Vc build), 1: S=float, A=double (non-Vc build),
prec 2: S=A=double (FP64 oracle).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libo3d_oracle.so")
# the same source built as the reference's Release build optimises (-O3, CMakeLists.txt:60,
# with the compiler's default contraction of multiply-adds; -march=native is left out, host
# code here builds the same on every machine): only a timing baseline, not bit-exact
FAST_PATH = os.path.join(HERE, "libo3d_oracle_o3.so")
REF_DIR = os.path.join(HERE, "_ref")

CORES = {"rm": 0, "wl": 1, "exp": 2, "gauss": 3, "v2": 4}
REF_CORES = ("rm", "wl", "exp", "v2")   # cores the reference itself implements

_lib = None
_ref = {}


def build_oracle(force=False):
    """Compile oracle/o3d_oracle.cpp into oracle/libo3d_oracle.so (the checker: -O2, no
    contraction, bit for bit the reference build's arithmetic) and libo3d_oracle_o3.so (the
    timing baseline at the reference's Release optimisation)."""
    src = os.path.join(HERE, "o3d_oracle.cpp")
    for path, flags in ((LIB_PATH, ["-O2", "-ffp-contract=off"]), (FAST_PATH, ["-O3"])):
        if (not force and os.path.exists(path) and os.path.getmtime(path) >= os.path.getmtime(src)):
            continue
        cmd = ["g++", "-std=c++17"] + flags + ["-fopenmp", "-fPIC", "-shared", src, "-o", path]
        subprocess.run(cmd, check=True)
    return LIB_PATH


def build_ref():
    """Compile the reference's own kernels into oracle/_ref (no-op without the sources)."""
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True)


def lib(fast=False):
    global _lib
    if fast:
        if "o3" not in _ref:
            build_oracle()
            _ref["o3"] = ctypes.CDLL(FAST_PATH)
        return _ref["o3"]
    if _lib is None:
        build_oracle()
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def ref_available(core="rm"):
    return os.path.exists(os.path.join(REF_DIR, "libo3dref_%s.so" % core))


def ref_lib(core):
    if core not in _ref:
        path = os.path.join(REF_DIR, "libo3dref_%s.so" % core)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        _ref[core] = ctypes.CDLL(path)
    return _ref[core]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _dtypes(prec):
    return np.float64 if prec == 2 else np.float32


def _as(a, dt):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=dt)


def _nthreads(nthreads):
    return int(nthreads) if nthreads else (os.cpu_count() or 1)


def points_affect_points(src_x, src_r, src_s, targ_x, targ_r=None, grads=True, core="rm", prec=0,
                         nthreads=0, use_ref=False, fast=False):
    """Returns (u[3,nt], ug[9,nt] or None) accumulated from zero.  fast: the -O3 build
    (timing baseline; not bit-exact)."""
    dt = _dtypes(prec)
    sx, sr, ss = _as(src_x, dt), _as(src_r, dt), _as(src_s, dt)
    tx, tr = _as(targ_x, dt), _as(targ_r, dt)
    ns, nt = sr.shape[0], tx.shape[1]
    tu = np.zeros((3, nt), dt)
    tug = np.zeros((9, nt), dt) if grads else None
    if use_ref:
        rc = ref_lib(core).ref_points_affect_points(
            ctypes.c_int(prec), ctypes.c_int(ns), _p(sx), _p(sr), _p(ss), ctypes.c_int(nt), _p(tx), _p(tr),
            _p(tu), _p(tug))
    else:
        rc = lib(fast).o3o_points_affect_points(
            ctypes.c_int(prec), ctypes.c_int(CORES[core]), ctypes.c_int(ns), _p(sx), _p(sr), _p(ss),
            ctypes.c_int(nt), _p(tx), _p(tr), _p(tu), _p(tug), ctypes.c_int(_nthreads(nthreads)))
    if rc != 0:
        raise RuntimeError("oracle points_affect_points failed")
    return tu, tug


def panels_affect_points(nodes, idx, area, ts, targ_x, sss=None, grads=True, core="rm", prec=0, maxlev=3,
                         nthreads=0, use_ref=False):
    dt = _dtypes(prec)
    nx, ar, t, tx, s3 = _as(nodes, dt), _as(area, dt), _as(ts, dt), _as(targ_x, dt), _as(sss, dt)
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    nn, np_, nt = nx.shape[1], ar.shape[0], tx.shape[1]
    tu = np.zeros((3, nt), dt)
    tug = np.zeros((9, nt), dt) if grads else None
    if use_ref:
        rc = ref_lib(core).ref_panels_affect_points(
            ctypes.c_int(prec), ctypes.c_int(maxlev), ctypes.c_int(nn), _p(nx), ctypes.c_int(np_), _p(idx),
            _p(ar), _p(t), _p(s3), ctypes.c_int(nt), _p(tx), _p(tu), _p(tug))
    else:
        rc = lib().o3o_panels_affect_points(
            ctypes.c_int(prec), ctypes.c_int(CORES[core]), ctypes.c_int(maxlev), ctypes.c_int(nn), _p(nx),
            ctypes.c_int(np_), _p(idx), _p(ar), _p(t), _p(s3), ctypes.c_int(nt), _p(tx), _p(tu), _p(tug),
            ctypes.c_int(_nthreads(nthreads)))
    if rc != 0:
        raise RuntimeError("oracle panels_affect_points failed")
    return tu, tug


def points_affect_panels(src_x, src_s, nodes, idx, area, core="rm", prec=0, maxlev=3, nthreads=0, use_ref=False):
    """Returns the (negated, reference convention) panel velocities pu[3, np] from zero."""
    dt = _dtypes(prec)
    sx, ss, nx, ar = _as(src_x, dt), _as(src_s, dt), _as(nodes, dt), _as(area, dt)
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    ns, nn, np_ = sx.shape[1], nx.shape[1], ar.shape[0]
    pu = np.zeros((3, np_), dt)
    if use_ref:
        rc = ref_lib(core).ref_points_affect_panels(
            ctypes.c_int(prec), ctypes.c_int(maxlev), ctypes.c_int(ns), _p(sx), _p(ss), ctypes.c_int(nn), _p(nx),
            ctypes.c_int(np_), _p(idx), _p(ar), _p(pu))
    else:
        rc = lib().o3o_points_affect_panels(
            ctypes.c_int(prec), ctypes.c_int(CORES[core]), ctypes.c_int(maxlev), ctypes.c_int(ns), _p(sx), _p(ss),
            ctypes.c_int(nn), _p(nx), ctypes.c_int(np_), _p(idx), _p(ar), _p(pu), ctypes.c_int(_nthreads(nthreads)))
    if rc != 0:
        raise RuntimeError("oracle points_affect_panels failed")
    return pu


def panels_on_panels_coeff(src, targ, nunk=2, is_self=True, core="rm", prec=0, maxlev=3, nthreads=0,
                           use_ref=False):
    """src/targ: dicts with nodes[3,nn], idx[np*3], area[np], x1[3,np], x2[3,np], norm[3,np].
    Returns the column-major block as a (ncols, nrows) array (row index fastest)."""
    dt = _dtypes(prec)
    S = {k: (_as(v, dt) if k != "idx" else np.ascontiguousarray(v, np.uint32)) for k, v in src.items()}
    T = {k: (_as(v, dt) if k != "idx" else np.ascontiguousarray(v, np.uint32)) for k, v in targ.items()}
    snp, tnp = S["area"].shape[0], T["area"].shape[0]
    out = np.zeros((snp * nunk, tnp * nunk), dt)
    args = [ctypes.c_int(maxlev), ctypes.c_int(nunk), ctypes.c_int(1 if is_self else 0),
            ctypes.c_int(S["nodes"].shape[1]), _p(S["nodes"]), ctypes.c_int(snp), _p(S["idx"]), _p(S["area"]),
            _p(S["x1"]), _p(S["x2"]),
            ctypes.c_int(T["nodes"].shape[1]), _p(T["nodes"]), ctypes.c_int(tnp), _p(T["idx"]), _p(T["area"]),
            _p(T["x1"]), _p(T["x2"]), _p(T["norm"]), _p(out)]
    if use_ref:
        rc = ref_lib(core).ref_panels_on_panels_coeff(ctypes.c_int(prec), *args)
    else:
        rc = lib().o3o_panels_on_panels_coeff(ctypes.c_int(prec), ctypes.c_int(CORES[core]), *args,
                                              ctypes.c_int(_nthreads(nthreads)))
    if rc != 0:
        raise RuntimeError("oracle panels_on_panels_coeff failed")
    return out


def compute_bases(nodes, idx):
    nx = _as(nodes, np.float32)
    idx = np.ascontiguousarray(idx, np.uint32)
    np_ = idx.shape[0] // 3
    x1, x2, nm = (np.zeros((3, np_), np.float32) for _ in range(3))
    area = np.zeros(np_, np.float32)
    rc = lib().o3o_compute_bases(ctypes.c_int(nx.shape[1]), _p(nx), ctypes.c_int(np_), _p(idx),
                                 _p(x1), _p(x2), _p(nm), _p(area))
    if rc != 0:
        raise RuntimeError("oracle compute_bases failed")
    return x1, x2, nm, area


def sheet_to_panel_strength(ps0, ps1, x1, x2, area):
    np_ = area.shape[0]
    ts = np.zeros((3, np_), np.float32)
    args = [_as(ps0, np.float32), _as(ps1, np.float32), _as(x1, np.float32), _as(x2, np.float32),
            _as(area, np.float32)]
    rc = lib().o3o_sheet_to_panel_strength(ctypes.c_int(np_), *[_p(a) for a in args], _p(ts))
    if rc != 0:
        raise RuntimeError("oracle sheet_to_panel_strength failed")
    return ts


def vels_to_rhs_panels(pu, x1, x2, norm, nunk=2):
    np_ = pu.shape[1]
    rhs = np.zeros(np_ * nunk, np.float32)
    args = [_as(pu, np.float32), _as(x1, np.float32), _as(x2, np.float32), _as(norm, np.float32)]
    rc = lib().o3o_vels_to_rhs_panels(ctypes.c_int(np_), ctypes.c_int(nunk), *[_p(a) for a in args], _p(rhs))
    if rc != 0:
        raise RuntimeError("oracle vels_to_rhs_panels failed")
    return rhs


def finalize_vels(u, ug, fs=(0.0, 0.0, 0.0)):
    """In place: u = fs + u/(4 pi) (double arithmetic), ug *= float(1/(4 pi))."""
    fsa = np.ascontiguousarray(fs, np.float64)
    rc = lib().o3o_finalize_vels(ctypes.c_int(u.shape[1]), _p(fsa), _p(u), _p(ug))
    if rc != 0:
        raise RuntimeError("oracle finalize_vels failed")


def points_move_euler(x, s, elong, u, ug, dt, wt1=1.0):
    rc = lib().o3o_points_move_euler(ctypes.c_int(x.shape[1]), ctypes.c_double(dt), ctypes.c_double(wt1),
                                     _p(x), _p(s), _p(elong), _p(u), _p(ug))
    if rc != 0:
        raise RuntimeError("oracle points_move_euler failed")


def points_move_rk2(x, s, elong, u1, ug1, u2, ug2, dt, wt1=0.25, wt2=0.75):
    rc = lib().o3o_points_move_rk2(ctypes.c_int(x.shape[1]), ctypes.c_double(dt), ctypes.c_double(wt1),
                                   _p(u1), _p(ug1), ctypes.c_double(wt2), _p(u2), _p(ug2), _p(x), _p(s),
                                   _p(elong))
    if rc != 0:
        raise RuntimeError("oracle points_move_rk2 failed")


def ref_ovoid_available():
    return os.path.exists(os.path.join(REF_DIR, "libo3dref_ovoid.so"))


def generate_ovoid(levels, rx=1.0, ry=1.0, rz=1.0, use_ref=False):
    """The icosahedral sphere of generate_ovoid (GeomHelper.cpp:41-91) refined `levels`
    times with igl upsample numbering (IglRefine.cpp, lib/igl/upsample.cpp), scaled by
    (rx, ry, rz): nodes (3, 10*4^L+2) float32 and panel node triples (3*20*4^L,) uint32.
    use_ref runs the reference's own code (oracle/_ref/libo3dref_ovoid.so)."""
    nn, np_ = 10 * 4 ** levels + 2, 20 * 4 ** levels
    idx = np.zeros(3 * np_, np.uint32)
    if use_ref:
        if "ovoid" not in _ref:
            _ref["ovoid"] = ctypes.CDLL(os.path.join(REF_DIR, "libo3dref_ovoid.so"))
        xi = np.zeros(3 * nn, np.float32)
        rc = _ref["ovoid"].ref_generate_ovoid(ctypes.c_int(levels), ctypes.c_float(rx), ctypes.c_float(ry),
                                              ctypes.c_float(rz), _p(xi), _p(idx))
        if rc != 0:
            raise RuntimeError("reference generate_ovoid failed")
        return np.ascontiguousarray(xi.reshape(nn, 3).T), idx
    x = np.zeros((3, nn), np.float32)
    rc = lib().o3o_generate_ovoid(ctypes.c_int(levels), ctypes.c_float(rx), ctypes.c_float(ry),
                                  ctypes.c_float(rz), _p(x), _p(idx))
    if rc != 0:
        raise RuntimeError("oracle generate_ovoid failed")
    return x, idx


def flops_per_pair(core="rm", grads=True, have_tr=True):
    return int(lib().o3o_flops_per_pair(ctypes.c_int(CORES[core]), ctypes.c_int(int(grads)),
                                        ctypes.c_int(int(have_tr))))


def ralston_step(x, s, r, elong, dt, core="rm", prec=1, fs=(0.0, 0.0, 0.0), nthreads=0):
    """One inviscid, boundary-free Ralston RK2 step of a particle set (Convection.h:349-425):
    returns new (x, s, elong) plus the stage-1 (u, ug) evaluated at the starting state."""
    x0, s0, e0 = x.copy(), s.copy(), elong.copy()
    u1, ug1 = points_affect_points(x0, r, s0, x0, r, True, core, prec, nthreads)
    u1, ug1 = u1.astype(np.float32), ug1.astype(np.float32)
    finalize_vels(u1, ug1, fs)
    xi, si, ei = x0.copy(), s0.copy(), e0.copy()
    points_move_euler(xi, si, ei, u1, ug1, 2.0 / 3.0 * dt, 1.0)
    u2, ug2 = points_affect_points(xi, r, si, xi, r, True, core, prec, nthreads)
    u2, ug2 = u2.astype(np.float32), ug2.astype(np.float32)
    finalize_vels(u2, ug2, fs)
    uc = u1.copy()
    points_move_rk2(x0, s0, e0, uc, ug1, u2, ug2, dt, 0.25, 0.75)
    return x0, s0, e0, u1, ug1


def solve_bem_body(x, s, body, A64, nunk, fs, core="rm", prec=1, maxlev=3):
    """solve_bem (BEMHelper.h:43-265) for one fixed body and one particle set: panel velocities
    from the particles (points_affect_panels, Influence.h:1107-1221, velocity only), freestream
    (finalize_vels, ElementBase.h:187-193), vels_to_rhs_panels (RHS.h:92-110), the system
    solved in FP64 with the matrix A64 (rows = targets), and Surfaces::set_str
    (Surfaces.h:267-335).  body: dict with nodes, idx, area, x1, x2, norm.
    Returns (ts[3, np], sss[np] or None, solution)."""
    pu = points_affect_panels(x, s, body["nodes"], body["idx"], body["area"], core, prec, maxlev)
    pu = pu.astype(np.float32)
    finalize_vels(pu, None, fs)
    rhs = vels_to_rhs_panels(pu, body["x1"], body["x2"], body["norm"], nunk)
    sol = np.linalg.solve(A64, rhs.astype(np.float64)).astype(np.float32)
    ts = sheet_to_panel_strength(sol[0::nunk], sol[1::nunk], body["x1"], body["x2"], body["area"])
    sss = np.ascontiguousarray(sol[2::nunk]) if nunk == 3 else None
    return ts, sss, sol


def coupled_ralston_step(x, s, r, elong, body, A64, nunk, dt, fs=(1.0, 0.0, 0.0), core="rm", prec=1, maxlev=3,
                         ips=0.0):
    """One Ralston RK2 step of vortex particles around one fixed body (Convection.h:349-425
    with find_derivs, Convection.h:188-202): at each stage the BEM is solved for the stage's
    particles, then velocity + gradient = particles (points_affect_points) + panels
    (panels_affect_points), each summed into float like the reference's += of per-call
    accumulators, then finalize_vels.  With ips > 0 the interim and the final positions are
    pushed out of the body (clear_inner_layer method 1, cutoff 0.5/sqrt(2 pi) * ips,
    Convection.h:372,423).  Returns new (x, s, elong) and the stage-2 solution."""
    cut = float(np.float32(0.5 / np.sqrt(2.0 * np.pi)))
    def derivs(xs, ss):
        ts, sss, sol = solve_bem_body(xs, ss, body, A64, nunk, fs, core, prec, maxlev)
        u, ug = points_affect_points(xs, r, ss, xs, r, True, core, prec)
        u, ug = u.astype(np.float32), ug.astype(np.float32)
        up, gp = panels_affect_points(body["nodes"], body["idx"], body["area"], ts, xs, sss, True, core, prec,
                                      maxlev)
        u = (u + up.astype(np.float32)).astype(np.float32)
        ug = (ug + gp.astype(np.float32)).astype(np.float32)
        finalize_vels(u, ug, fs)
        return u, ug, sol
    x0, s0, e0 = x.copy(), s.copy(), elong.copy()
    u1, ug1, _ = derivs(x0, s0)
    xi, si, ei = x0.copy(), s0.copy(), e0.copy()
    points_move_euler(xi, si, ei, u1, ug1, 2.0 / 3.0 * dt, 1.0)
    if ips > 0:
        clear_inner_layer(xi, body["nodes"], body["idx"], body["norm"], cut, ips)
    u2, ug2, sol2 = derivs(xi, si)
    uc = u1.copy()
    points_move_rk2(x0, s0, e0, uc, ug1, u2, ug2, dt, 0.25, 0.75)
    if ips > 0:
        clear_inner_layer(x0, body["nodes"], body["idx"], body["norm"], cut, ips)
    return x0, s0, e0, sol2


def clear_inner_layer(x, nodes, idx, norm, cutoff_mult=0.5 / np.sqrt(2.0 * np.pi), ips=0.01, prec=0, nthreads=0,
                      use_ref=False):
    """clear_inner_layer method 1 (Reflect.h:446-656) in place on x[3, n]: points below the
    cutoff layer (cutoff_mult * ips above the closest panels) are pushed out along the mean
    normal of the closest panels.  Returns the number of points pushed."""
    dt = np.float64 if prec == 2 else np.float32
    assert x.dtype == dt and x.flags["C_CONTIGUOUS"]
    nx, nm = _as(nodes, dt), _as(norm, dt)
    idx = np.ascontiguousarray(idx, np.uint32)
    n, nn, np_ = x.shape[1], nx.shape[1], nm.shape[1]
    if use_ref:
        path = os.path.join(REF_DIR, "libo3dref_reflect.so")
        if "reflect" not in _ref:
            _ref["reflect"] = ctypes.CDLL(path)
        rc = _ref["reflect"].ref_clear_inner_layer(ctypes.c_int(prec), ctypes.c_int(n), _p(x), ctypes.c_int(nn),
                                                   _p(nx), ctypes.c_int(np_), _p(idx), _p(nm),
                                                   ctypes.c_double(cutoff_mult), ctypes.c_double(ips))
    else:
        rc = lib().o3o_clear_inner_layer(ctypes.c_int(prec), ctypes.c_int(n), _p(x), ctypes.c_int(nn), _p(nx),
                                         ctypes.c_int(np_), _p(idx), _p(nm), ctypes.c_double(cutoff_mult),
                                         ctypes.c_double(ips), ctypes.c_int(_nthreads(nthreads)))
    if rc < 0:
        raise RuntimeError("oracle clear_inner_layer failed")
    return int(rc)


def ref_reflect_available():
    return os.path.exists(os.path.join(REF_DIR, "libo3dref_reflect.so"))


def represent_as_particles(nodes, idx, area, x1, x2, norm, offset, ts, bc1=None, bc2=None):
    """Surfaces::represent_as_particles (Surfaces.h:959-1008): (positions[3, np],
    strengths[3, np]) of one particle per panel."""
    nx = _as(nodes, np.float32)
    idx = np.ascontiguousarray(idx, np.uint32)
    np_ = area.shape[0]
    px = np.zeros((3, np_), np.float32)
    ps = np.zeros((3, np_), np.float32)
    arrs = [_as(a, np.float32) for a in (area, x1, x2, norm, ts)]
    b1 = _as(bc1, np.float32)
    b2 = _as(bc2, np.float32)
    rc = lib().o3o_represent_as_particles(ctypes.c_int(nx.shape[1]), _p(nx), ctypes.c_int(np_), _p(idx),
                                          _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
                                          ctypes.c_float(offset), _p(arrs[4]), _p(b1), _p(b2), _p(px), _p(ps))
    if rc != 0:
        raise RuntimeError("oracle represent_as_particles failed")
    return px, ps


def ref_splitmerge_available():
    return os.path.exists(os.path.join(REF_DIR, "libo3dref_splitmerge.so"))


def _splitmerge_lib(use_ref):
    if not use_ref:
        return lib(), "o3o_"
    if "splitmerge" not in _ref:
        _ref["splitmerge"] = ctypes.CDLL(os.path.join(REF_DIR, "libo3dref_splitmerge.so"))
    return _ref["splitmerge"], "ref_"


def _tie_args(use_ref, tie_order):
    """The oracle's trailing tie_order argument: 0 visits equal-distance neighbours in
    increasing index (the kernels' order), 1 in the order of the restated nanoflann kd-tree
    (the reference's).  The reference build has no such argument."""
    if tie_order not in ("index", "kdtree"):
        raise ValueError("tie_order must be 'index' or 'kdtree'")
    return () if use_ref else (ctypes.c_int(int(tie_order == "kdtree")),)


def split_elongated(x, s, r, elong, core=0, overlap=1.5, threshold=1.2, use_ref=False, tie_order="index"):
    """split_elongated<float> (Split.h:44-270) on x[3, n], s[3, n], r[n], elong[n]
    (core 0 = gaussian, 1 = compactg, Core.h:27).  Returns new arrays
    (x, s, r, elong) of n + nsplit particles (children appended in index order) and nsplit.
    tie_order: see _tie_args."""
    n = x.shape[1]
    m = int(np.count_nonzero(np.asarray(elong, np.float32) > np.float32(threshold)))
    cap = n + m
    xs = np.zeros((3, cap), np.float32)
    ss = np.zeros((3, cap), np.float32)
    rs = np.zeros(cap, np.float32)
    es = np.zeros(cap, np.float32)
    xs[:, :n], ss[:, :n], rs[:n], es[:n] = x, s, r, elong
    L, pre = _splitmerge_lib(use_ref)
    rc = getattr(L, pre + "split_elongated")(
        ctypes.c_int(n), ctypes.c_int(cap), _p(xs[0]), _p(xs[1]), _p(xs[2]), _p(rs), _p(es), _p(ss[0]), _p(ss[1]),
        _p(ss[2]), ctypes.c_int(core), ctypes.c_float(overlap), ctypes.c_float(threshold),
        *_tie_args(use_ref, tie_order))
    if rc < 0:
        raise RuntimeError("split_elongated failed")
    assert rc == m
    return xs, ss, rs, es, rc


def merge_close_particles(x, s, r, overlap=1.5, threshold=0.2, adapt_radii=False, use_ref=False,
                          tie_order="index"):
    """merge_close_particles<float> (Merge.h:45-218) on x[3, n], s[3, n], r[n].  Returns
    new arrays (x, s, r) of the survivors in their original order and the number removed.
    tie_order: see _tie_args."""
    n = x.shape[1]
    xs = np.array(x, np.float32, order="C", copy=True)
    ss = np.array(s, np.float32, order="C", copy=True)
    rs = np.array(r, np.float32, copy=True)
    L, pre = _splitmerge_lib(use_ref)
    rc = getattr(L, pre + "merge_close_particles")(
        ctypes.c_int(n), _p(xs[0]), _p(xs[1]), _p(xs[2]), _p(ss[0]), _p(ss[1]), _p(ss[2]), _p(rs),
        ctypes.c_float(overlap), ctypes.c_float(threshold), ctypes.c_int(int(bool(adapt_radii))),
        *_tie_args(use_ref, tie_order))
    if rc < 0:
        raise RuntimeError("merge_close_particles failed")
    k = n - rc
    return np.ascontiguousarray(xs[:, :k]), np.ascontiguousarray(ss[:, :k]), rs[:k].copy(), rc


def gmres_restarted(A, b, restart=30, tol=None, max_iter=None):
    """Restated restarted GMRES of Eigen::GMRES, the solver BEM<S,I>::solve uses
    (BEM.h:182-202, third-party Eigen >= 3.3, not vendored): left diagonal (Jacobi)
    preconditioner with 1 where the diagonal is zero, restart 30, tolerance = epsilon of the
    matrix's type, at most 2n iterations, all in the matrix's precision.  A: (n, n) array
    (any layout numpy can multiply); b: (n,).  Returns (x, iterations, relative residual of
    the unpreconditioned system).  Timed by bench.py as the CPU baseline of the BEM solve."""
    dt = A.dtype
    n = b.shape[0]
    tol = np.finfo(dt).eps if tol is None else tol
    max_iter = 2 * n if max_iter is None else max_iter
    d = np.ascontiguousarray(np.diagonal(A)).astype(dt)
    inv = np.where(d != 0, 1 / np.where(d != 0, d, 1), 1).astype(dt)
    b = b.astype(dt)
    x = np.zeros(n, dt)
    pb = np.linalg.norm(inv * b)
    if pb == 0:
        return x, 0, 0.0
    it = 0
    while it < max_iter:
        r = inv * (b - A @ x)
        beta = np.linalg.norm(r)
        if beta / pb <= tol:
            break
        m = min(restart, max_iter - it)
        V = np.zeros((m + 1, n), dt)
        H = np.zeros((m + 1, m), np.float64)
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        V[0] = r / beta
        k_done = 0
        for k in range(m):
            w = inv * (A @ V[k])
            for j in range(k + 1):              # modified Gram-Schmidt
                H[j, k] = float(V[j] @ w)
                w = w - dt.type(H[j, k]) * V[j]
            H[k + 1, k] = float(np.linalg.norm(w))
            if H[k + 1, k] != 0:
                V[k + 1] = w / dt.type(H[k + 1, k])
            for j in range(k):                  # previous Givens rotations
                h0, h1 = H[j, k], H[j + 1, k]
                H[j, k], H[j + 1, k] = cs[j] * h0 + sn[j] * h1, -sn[j] * h0 + cs[j] * h1
            den = np.hypot(H[k, k], H[k + 1, k])
            cs[k], sn[k] = (H[k, k] / den, H[k + 1, k] / den) if den != 0 else (1.0, 0.0)
            H[k, k], H[k + 1, k] = den, 0.0
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            it += 1
            k_done = k + 1
            if abs(g[k + 1]) / pb <= tol or H[k, k] == 0:
                break
        y = np.linalg.solve(np.triu(H[:k_done, :k_done]), g[:k_done])
        x = x + (V[:k_done].T @ y.astype(dt)).astype(dt)
    bn = np.linalg.norm(b.astype(np.float64))
    rel = float(np.linalg.norm(b.astype(np.float64) - A.astype(np.float64) @ x.astype(np.float64)) / bn)
    return x, it, rel


# ---- the reference's VTU writer (oracle/_ref/libo3dref_vtk.so) -------------------------
def ref_vtk_available():
    return os.path.exists(os.path.join(REF_DIR, "libo3dref_vtk.so"))


def _vtk_lib():
    if "vtk" not in _ref:
        path = os.path.join(REF_DIR, "libo3dref_vtk.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle/_ref/libo3dref_vtk.so missing: run sh oracle/build_ref.sh")
        _ref["vtk"] = ctypes.CDLL(path)
    return _ref["vtk"]


def ref_write_points_vtu(path, x, u, s=None, r=None, time=0.0):
    """The reference's VtkXmlWriter driven as Points::write_vtk drives it (Points.h:851-1039):
    particles with strengths s[3, n] and radii r[n], or field points (s, r None)."""
    f = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    x, u = f(x), f(u)
    n = x.shape[1]
    if s is not None:
        s, r = f(s), f(r)
        sp = [_p(s[0]), _p(s[1]), _p(s[2])]
        rp = _p(r)
    else:
        sp, rp = [None] * 3, None
    rc = _vtk_lib().ref_write_points_vtu(path.encode(), ctypes.c_int(n), _p(x[0]), _p(x[1]), _p(x[2]), *sp, rp,
                                         _p(u[0]), _p(u[1]), _p(u[2]), ctypes.c_double(time))
    if rc != 0:
        raise RuntimeError("reference VTU writer failed")
    return path


def ref_write_panels_vtu(path, nodes, idx, sheet=None, src=None, time=0.0):
    """The reference's VtkXmlWriter driven as Surfaces::write_vtk drives it
    (Surfaces.h:1301-1458): triangles over the nodes, the vortex sheet vector per panel and
    the source sheet strength as cell data when given."""
    f = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    x = f(nodes)
    ix = np.ascontiguousarray(idx, np.uint32).reshape(-1)
    npan = ix.size // 3
    tp = [None] * 3
    if sheet is not None:
        sheet = f(sheet)
        tp = [_p(sheet[0]), _p(sheet[1]), _p(sheet[2])]
    sp = None
    if src is not None:
        src = f(src)
        sp = _p(src)
    rc = _vtk_lib().ref_write_panels_vtu(path.encode(), ctypes.c_int(x.shape[1]), _p(x[0]), _p(x[1]), _p(x[2]),
                                         ctypes.c_int(npan), _p(ix), *tp, sp, ctypes.c_double(time))
    if rc != 0:
        raise RuntimeError("reference VTU writer failed")
    return path
