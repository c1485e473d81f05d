"""Generates the golden vectors in tests/golden/ from the REFERENCE's own kernels.

Run in a checkout that has the reference sources (oracle/build_ref.sh compiles
src/Kernels.h, src/CoreFunc.h and src/MathHelper.h of the reference into
oracle/_ref/libo3dref_<core>.so, src/Reflect.h into oracle/_ref/libo3dref_reflect.so, and
src/Split.h + src/Merge.h with lib/nanoflann into oracle/_ref/libo3dref_splitmerge.so;
the loops around them are oracle/ref_driver.cpp, oracle/ref_reflect_driver.cpp and
oracle/ref_splitmerge_driver.cpp):

    sh oracle/build_ref.sh && python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py --only reflect                       # reflect.npz alone
    python tests/golden/make_golden.py --only splitmerge                    # splitmerge*.npz alone
    python tests/golden/make_golden.py --only edges                         # branch_edges.npz alone
    python tests/golden/make_golden.py --only vtk                           # vtk_files.npz alone

Every fixture holds its seeded inputs and the outputs of the reference build for the
precisions named in it:  prec 0 = S=A=float (Vc build semantics), prec 2 = S=A=double.
The Gaussian core has no reference implementation; its fixture comes from the oracle
restatement and is marked "pinned": False.  The sphere fixture comes from the reference's
generate_ovoid + igl upsample, built against oracle/eigen_shim_igl
(python tests/golden/make_golden.py --only sphere writes it alone).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from omega3d_gb300 import workloads as W  # noqa: E402


def _save(name, meta, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def pair_inputs():
    x, s, r = W.gaussian_cloud(192, seed=11, pos_std=0.2, rmin=0.02, rmax=0.06)
    tx2, _, tr2 = W.gaussian_cloud(96, seed=12, pos_std=0.25, rmin=0.02, rmax=0.06)
    # the first 64 targets coincide with sources (self pairs, d = 0)
    tx = np.concatenate([x[:, :64], tx2], axis=1)
    tr = np.concatenate([r[:64], tr2])
    return x, s, r, tx, tr


def sphere_inputs(levels=1, scale=2.0, seed=13):
    nodes, idx = O.generate_ovoid(levels, scale, scale, scale)
    x1, x2, nm, area = O.compute_bases(nodes, idx)
    rng = np.random.default_rng(seed)
    np_ = area.shape[0]
    ps0 = rng.normal(size=np_).astype(np.float32)
    ps1 = rng.normal(size=np_).astype(np.float32)
    sss = rng.normal(size=np_).astype(np.float32)
    ts = O.sheet_to_panel_strength(ps0, ps1, x1, x2, area)
    return dict(nodes=nodes, idx=idx, x1=x1, x2=x2, norm=nm, area=area, ps0=ps0, ps1=ps1, sss=sss, ts=ts)


def reflect_inputs(levels=2, scale=2.0, seed=15, n=1500):
    """Points around and inside a sphere, on its nodes and just inside them."""
    nodes, idx = O.generate_ovoid(levels, scale, scale, scale)
    x1, x2, nm, area = O.compute_bases(nodes, idx)
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(3, n))
    d /= np.linalg.norm(d, axis=0)
    pts = (d * rng.uniform(0.85, 1.06, n)).astype(np.float32)
    k = min(100, nodes.shape[1])
    pts = np.concatenate([pts, nodes[:, :k].copy(), (nodes[:, :k] * np.float32(0.995)).astype(np.float32)], axis=1)
    return dict(nodes=nodes, idx=idx, norm=nm), np.ascontiguousarray(pts)


def write_reflect():
    if not O.ref_reflect_available():
        raise SystemExit("oracle/_ref/libo3dref_reflect.so missing: run sh oracle/build_ref.sh")
    geo, pts = reflect_inputs()
    out = {}
    for prec in (0, 2):
        x = pts.astype(np.float64 if prec == 2 else np.float32).copy()
        out["npushed_p%d" % prec] = np.array(O.clear_inner_layer(x, geo["nodes"], geo["idx"], geo["norm"],
                                                                  ips=0.05, prec=prec, use_ref=True))
        out["x_p%d" % prec] = x
    _save("reflect.npz", {"pinned": True, "method": 1, "ips": 0.05, "cutoff_mult": "0.5/sqrt(2 pi)",
                          "source": "reference Reflect.h"}, x_in=pts, **geo, **out)


def write_splitmerge():
    """Split and merge of a jittered 12^3 lattice by the reference's own Split.h / Merge.h
    (oracle/_ref/libo3dref_splitmerge.so, with the vendored nanoflann)."""
    if not O.ref_splitmerge_available():
        raise SystemExit("oracle/_ref/libo3dref_splitmerge.so missing: run sh oracle/build_ref.sh")
    x, s, r, e = W.lattice_particles(k=12, seed=16)
    out = {}
    for core in (0, 1):
        xs, ss, rs, es, m = O.split_elongated(x, s, r, e, core, 1.5, 1.2, use_ref=True)
        out.update({"split%d_x" % core: xs, "split%d_s" % core: ss, "split%d_r" % core: rs,
                    "split%d_e" % core: es})
    for name, thr, adapt in (("merge_vrm", 0.2, False), ("merge_core", 0.02, False), ("merge_amr", 0.2, True)):
        xm, sm, rm, nrem = O.merge_close_particles(x, s, r, 1.5, thr, adapt, use_ref=True)
        out.update({name + "_x": xm, name + "_s": sm, name + "_r": rm})
    _save("splitmerge.npz", {"pinned": True, "overlap": 1.5, "split_threshold": 1.2,
                             "merge": {"merge_vrm": [0.2, False], "merge_core": [0.02, False],
                                       "merge_amr": [0.2, True]},
                             "source": "reference Split.h / Merge.h with lib/nanoflann"},
          x_in=x, s_in=s, r_in=r, e_in=e, **out)
    write_splitmerge_tied()


def write_splitmerge_tied():
    """Inputs with neighbours at exactly equal float distances, where the reference's
    visiting order of the ties comes from its nanoflann kd-tree and std::sort: the split of
    an unjittered 12^3 lattice (Split.h) and the merge of a lattice with duplicated particles
    (Merge.h)."""
    x, s, r, e = W.lattice_particles(k=12, seed=40, jitter=0.0)
    out = {}
    for core in (0, 1):
        xs, ss, rs, es, m = O.split_elongated(x, s, r, e, core, 1.5, 1.2, use_ref=True)
        out.update({"split%d_x" % core: xs, "split%d_s" % core: ss, "split%d_r" % core: rs,
                    "split%d_e" % core: es})
    xd, sd, rd, _ = W.duplicated_particles(k=12, seed=41, every=5, seed_dup=2)
    for name, thr in (("merge_vrm", 0.2), ("merge_core", 0.02)):
        xm, sm, rm, nrem = O.merge_close_particles(xd, sd, rd, 1.5, thr, False, use_ref=True)
        out.update({name + "_x": xm, name + "_s": sm, name + "_r": rm})
    _save("splitmerge_tied.npz", {"pinned": True, "overlap": 1.5, "split_threshold": 1.2,
                                  "merge": {"merge_vrm": 0.2, "merge_core": 0.02},
                                  "source": "reference Split.h / Merge.h with lib/nanoflann"},
          x_in=x, s_in=s, r_in=r, e_in=e, xd_in=xd, sd_in=sd, rd_in=rd, **out)


def branch_edge_inputs():
    """One source at the origin and targets where the cores switch form: d^3/sigma^3 just
    below, at and above 0.001 and 16 (the exponential core's branches, CoreFunc.h:119-177)
    and 332.55 (q = d^2/sigma^2 = 48, the Gaussian core's far-field switch), d = 0, and
    d^3/sigma^3 from 1e-12 to 1e9, each in 4 random directions.  Particle targets carry
    sigma_t = sigma_s, so their combined core is 2 sigma^3 (EXP) or 2 sigma^2; field points
    have sigma_s alone.  Returns the inputs and, per target kind, the d^3/sigma^3 values."""
    rng = np.random.default_rng(37)
    sig = np.float32(0.05)
    rel = np.array([0.0] + [v * f for v in (1e-3, 16.0, 332.55) for f in (0.999, 1.0, 1.001)]
                   + [1e-12, 1e-9, 1e-6, 0.1, 1.0, 4.0, 1e3, 1e9])
    rel = np.repeat(rel, 4)
    d = rng.normal(size=(3, rel.size))
    d /= np.linalg.norm(d, axis=0)
    sx = np.zeros((3, 1), np.float32)
    ss = np.array([[0.3], [-0.2], [0.5]], np.float32)
    sr = np.array([sig], np.float32)
    tr = np.full(rel.size, sig, np.float32)
    tx_p = (d * np.cbrt(rel * 2.0 * float(sig) ** 3)).astype(np.float32)
    tx_f = (d * np.cbrt(rel * float(sig) ** 3)).astype(np.float32)
    return dict(sx=sx, ss=ss, sr=sr, tr=tr, tx_p=tx_p, tx_f=tx_f, rel=rel)


def write_branch_edges():
    """Per-pair outputs at the cores' branch edges from the reference kernels (RM, WL, EXP,
    V2; the Gaussian core from the oracle restatement) at prec 0 and 2."""
    for core in O.REF_CORES:
        if not O.ref_available(core):
            raise SystemExit("oracle/_ref/libo3dref_%s.so missing: run sh oracle/build_ref.sh" % core)
    inp = branch_edge_inputs()
    out = {}
    for core in ("rm", "wl", "exp", "v2", "gauss"):
        use_ref = core != "gauss"
        for prec in (0, 2):
            for tag, tx, tr in (("pg", inp["tx_p"], inp["tr"]), ("fg", inp["tx_f"], None)):
                u, g = O.points_affect_points(inp["sx"], inp["sr"], inp["ss"], tx, tr, True, core, prec,
                                              use_ref=use_ref)
                out["%s_%s_u_p%d" % (core, tag, prec)], out["%s_%s_g_p%d" % (core, tag, prec)] = u, g
            u, _ = O.points_affect_points(inp["sx"], inp["sr"], inp["ss"], inp["tx_p"], inp["tr"], False, core,
                                          prec, use_ref=use_ref)
            out["%s_pv_u_p%d" % (core, prec)] = u
    _save("branch_edges.npz", {"pinned": {c: c != "gauss" for c in ("rm", "wl", "exp", "v2", "gauss")},
                               "source": "reference kernels (gauss: oracle restatement)"}, **inp, **out)


def vtk_inputs():
    """Seeded particles, field points and a level-1 sphere's panels with sheet strengths."""
    rng = np.random.default_rng(38)
    n, nf = 37, 11
    x = rng.normal(size=(3, n)).astype(np.float32)
    s = rng.normal(size=(3, n)).astype(np.float32)
    r = rng.uniform(0.01, 0.05, n).astype(np.float32)
    u = rng.normal(size=(3, n)).astype(np.float32)
    fx = rng.normal(size=(3, nf)).astype(np.float32)
    fu = rng.normal(size=(3, nf)).astype(np.float32)
    nodes, idx = O.generate_ovoid(1, 2.0, 2.0, 2.0)
    npan = idx.size // 3
    sheet = rng.normal(size=(3, npan)).astype(np.float32)
    src = rng.normal(size=npan).astype(np.float32)
    return dict(x=x, s=s, r=r, u=u, fx=fx, fu=fu, nodes=nodes, idx=idx, sheet=sheet, src=src)


def write_vtk_golden():
    """Files written by the reference's own VtkXmlWriter (oracle/_ref/libo3dref_vtk.so),
    driven as Points::write_vtk and Surfaces::write_vtk drive it, stored as bytes."""
    import tempfile
    if not O.ref_vtk_available():
        raise SystemExit("oracle/_ref/libo3dref_vtk.so missing: run sh oracle/build_ref.sh")
    d = vtk_inputs()
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "f.vtu")
        for name, call in (("part", lambda: O.ref_write_points_vtu(f, d["x"], d["u"], d["s"], d["r"], 2.5)),
                           ("fldpt", lambda: O.ref_write_points_vtu(f, d["fx"], d["fu"], None, None, 0.125)),
                           ("panel3", lambda: O.ref_write_panels_vtu(f, d["nodes"], d["idx"], d["sheet"], d["src"],
                                                                    1.0)),
                           ("panel2", lambda: O.ref_write_panels_vtu(f, d["nodes"], d["idx"], d["sheet"], None, 1.0))):
            call()
            out[name] = np.frombuffer(open(f, "rb").read(), np.uint8)
    _save("vtk_files.npz", {"pinned": True, "source": "reference VtkXmlWriter.h with lib/tinyxml2, lib/cppcodec",
                            "times": {"part": 2.5, "fldpt": 0.125, "panel3": 1.0, "panel2": 1.0}}, **d, **out)


def main():
    if "--only" in sys.argv and sys.argv[-1] == "vtk":
        write_vtk_golden()
        return
    if "--only" in sys.argv and sys.argv[-1] == "edges":
        write_branch_edges()
        return
    if "--only" in sys.argv and sys.argv[-1] == "reflect":
        write_reflect()
        return
    if "--only" in sys.argv and sys.argv[-1] == "splitmerge":
        write_splitmerge()
        return
    if "--only" in sys.argv and sys.argv[-1] == "sphere":
        write_sphere()
        return
    for core in O.REF_CORES:
        if not O.ref_available(core):
            raise SystemExit("oracle/_ref/libo3dref_%s.so missing: run sh oracle/build_ref.sh" % core)
    x, s, r, tx, tr = pair_inputs()
    for core in ("rm", "wl", "exp", "v2", "gauss"):
        use_ref = core != "gauss"
        out = {}
        for prec in (0, 2):
            u, g = O.points_affect_points(x, r, s, tx, tr, True, core, prec, use_ref=use_ref)
            out["pg_u_p%d" % prec], out["pg_g_p%d" % prec] = u, g
            u, g = O.points_affect_points(x, r, s, tx, None, True, core, prec, use_ref=use_ref)
            out["fg_u_p%d" % prec], out["fg_g_p%d" % prec] = u, g
            u, _ = O.points_affect_points(x, r, s, tx, tr, False, core, prec, use_ref=use_ref)
            out["pv_u_p%d" % prec] = u
        _save("ptpt_%s.npz" % core, {"core": core, "pinned": use_ref, "source": "reference kernels" if use_ref
                                     else "oracle restatement"}, sx=x, ss=s, sr=r, tx=tx, tr=tr, **out)

    sph = sphere_inputs()
    ptx, pts, ptr = W.shell_particles(64, seed=14, rin=1.02, rout=1.5)
    ptx[:, :8] *= np.float32(1.0 / 1.1)   # a few targets close to the surface (subdivision active)
    for core in ("rm", "wl", "exp"):
        out = {}
        for prec in (0, 2):
            u, g = O.panels_affect_points(sph["nodes"], sph["idx"], sph["area"], sph["ts"], ptx, sph["sss"], True,
                                          core, prec, use_ref=True)
            out["pg_u_p%d" % prec], out["pg_g_p%d" % prec] = u, g
            u, _ = O.panels_affect_points(sph["nodes"], sph["idx"], sph["area"], sph["ts"], ptx, None, False, core,
                                          prec, use_ref=True)
            out["pv_u_p%d" % prec] = u
            out["pan_u_p%d" % prec] = O.points_affect_panels(ptx, pts, sph["nodes"], sph["idx"], sph["area"], core,
                                                             prec, use_ref=True)
        _save("panel_%s.npz" % core, {"core": core, "pinned": True, "maxlev": 3, "source": "reference kernels"},
              tx=ptx, ps=pts, **sph, **out)

    geo = {k: sph[k] for k in ("nodes", "idx", "area", "x1", "x2", "norm")}
    for core in ("rm", "wl"):
        out = {}
        for nunk in (2, 3):
            out["c%d_p0" % nunk] = O.panels_on_panels_coeff(geo, geo, nunk, True, core, 0, use_ref=True)
        if core == "rm":
            out["c2_p2"] = O.panels_on_panels_coeff(geo, geo, 2, True, core, 2, use_ref=True)
        _save("coeff_%s.npz" % core, {"core": core, "pinned": True, "maxlev": 3, "is_self": True,
                                      "source": "reference kernels"}, **geo, **out)

    write_sphere()
    write_reflect()
    write_splitmerge()
    write_branch_edges()
    write_vtk_golden()


def write_sphere():
    """The icosahedral sphere (levels 0-3, scale 2) from the reference's own generate_ovoid
    (src/GeomHelper.cpp) with refine_geometry (src/IglRefine.cpp) and the vendored igl
    upsample (oracle/_ref/libo3dref_ovoid.so)."""
    if not O.ref_ovoid_available():
        raise SystemExit("oracle/_ref/libo3dref_ovoid.so missing: run sh oracle/build_ref.sh")
    arrays = {}
    for lev in range(4):
        n, i = O.generate_ovoid(lev, 2.0, 2.0, 2.0, use_ref=True)
        arrays["nodes_L%d" % lev], arrays["idx_L%d" % lev] = n, i
    _save("sphere.npz", {"pinned": True, "scale": 2.0,
                         "source": "reference generate_ovoid + refine_geometry + igl upsample"}, **arrays)


if __name__ == "__main__":
    main()
