#!/usr/bin/env python
"""Benchmark: Biot-Savart velocity + velocity-gradient interactions/s on GB300.

Workload (one "step"): one direct-sum evaluation of velocity and the 9-component
velocity gradient at every particle of the precision cloud -- N = 262,144 particles,
positions N(0, 0.3^2) per axis, strength components N(0,1)*1e-3, core radii U[0.01,
0.03], Gaussian core, targets = sources (N^2 = 6.87e10 interactions including i = j).
Inputs are seeded synthetic data generated here.

value : interactions/s of the chosen form (COMPENSATED FP32) with inputs resident in
        HBM, device time per step from CUDA events on the launching stream; L2 is
        flushed (256 MiB write) between timed steps (inputs are 8 MiB, below L2).
e2e   : the same metric through the C-ABI with host (pinned) buffers: host->device
        copies, the sums and the device->host copy of the results in every step.
The plain FP32 drop-in path, the FP64 comparator on the same GPU, the errors of every
path against the FP64 sums, and the reference CPU baseline ride along in the line.

--impl reference times the reference's CPU algorithm for the same metric: the oracle
port (oracle/o3d_oracle.cpp: the reference's loops, float pair arithmetic with double
accumulators like its non-Vc build, OpenMP over targets) on the host's cores.
Multi-GPU (torchrun): every rank runs an independent replica ("replicas only": the
reference is single-GPU and this path has no data exchange); value sums the ranks'
interactions over the max time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Biot-Savart vel+grad interactions/s at stated FP64-oracle error"
# the metric's second half, "BEM solve time", is reported in the line's "bem_solve" object
UNIT = "interactions/s"
CORE = "gauss"
N_DEFAULT = 262144


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--core", default=CORE)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-bem", action="store_true")
    ap.add_argument("--skip-bem-fp64", action="store_true", help="skip the FP64 LU comparator (~50 s)")
    ap.add_argument("--bem-level", type=int, default=5,
                    help="sphere refinement levels of the BEM section (5: 20,480 panels; smaller for profiling)")
    ap.add_argument("--skip-ring", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--skip-splitmerge", action="store_true")
    ap.add_argument("--only", choices=["bem", "ring", "batch", "coupled", "splitmerge", "gemm"], default=None,
                    help="run one workload section alone and print its results (profiling)")
    ap.add_argument("--coupled-steps", type=int, default=2,
                    help="coupled sphere + 1M-particle Ralston steps to time (0 skips; 20 = the full run)")
    return ap.parse_args()


def whole_job(local_step_ms, units_per_rank, world, dist=None, device=None):
    """Replicas: every rank processes the same number of units; the job's rate is all ranks'
    units over the slowest rank's step time (all-reduce MAX).  Returns (units/s, max ms)."""
    step_max = float(local_step_ms)
    if world > 1:
        import torch
        t = torch.tensor([step_max], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_max = float(t.item())
    return world * units_per_rank / (step_max * 1e-3), step_max


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def config(args):
    return {"workload": "precision cloud: N=%d Gaussian-core particles, self-interaction vel+grad" % args.n,
            "n_particles": args.n, "core": args.core, "interactions_per_step": args.n * args.n,
            "targets_have_radius": True, "l2": "flushed between timed steps (256 MiB write); inputs 8 MiB",
            "seed": 2, "parallelism": "replicas"}


# ------------------------------------------------------------------------------------
def cpu_reference(args, nthreads=None, ntarg=None, reps=1, build=None):
    """Times the oracle port on a bounded sample: `ntarg` targets against all sources.
    build: "o3" (the reference's Release optimisation), "o2" (the bit-exact checker build),
    or None: both are timed on a first sample and the faster one is used."""
    import oracle
    from omega3d_gb300 import workloads as W
    x, s, r = W.gaussian_cloud(args.n, seed=2)
    nthreads = nthreads or (os.cpu_count() or 1)
    ntarg = ntarg or min(args.n, 8192)
    # a seeded subset of the targets, against all sources; scaled to the full count by rate
    idx = np.sort(np.random.default_rng(7).choice(args.n, ntarg, replace=False)).astype(np.int64)
    tx, tr = np.ascontiguousarray(x[:, idx]), np.ascontiguousarray(r[idx])

    def once(fast):
        t0 = time.perf_counter()
        oracle.points_affect_points(x, r, s, tx, tr, True, args.core, 1, nthreads, fast=fast)
        return time.perf_counter() - t0

    for fast in (False, True):
        oracle.points_affect_points(x[:, :4096], r[:4096], s[:, :4096], tx[:, :64], tr[:64], True, args.core, 1,
                                    nthreads, fast=fast)
    if build is None:
        build = "o3" if once(True) < once(False) else "o2"
    times = [once(build == "o3") for _ in range(reps)]
    pairs = float(ntarg) * args.n
    flags = "-O3" if build == "o3" else "-O2 -ffp-contract=off"
    return (pairs / statistics.median(times), nthreads,
            "%d targets x %d sources per sample (%.1f%% of the targets); port built %s" % (
                ntarg, args.n, 100.0 * ntarg / args.n, flags), times)


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    samples = []
    build = None
    for k in range(args.warmup + args.steps):
        v, cores, sample, _ = cpu_reference(args, build=build)
        build = "o3" if "-O3" in sample else "o2"
        if k >= args.warmup:
            samples.append(v)
    v = statistics.median(samples)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(args.n) * args.n / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (pairs) / f64 (accumulators)", "data": "synthetic",
            "config": config(args), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [c.strip() for c in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.remove(self.path)
        if not rows:
            return None
        sm = [float(f[1]) for f in rows if f[1].replace(".", "").isdigit()]
        mx = [float(f[2]) for f in rows if f[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for f in rows for i in range(4) if f[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def bem_rates(n, assemble_ms, factor_ms):
    """The assembly's rate against the HBM roof (it writes the n x n FP32 matrix once: 4 n^2
    algorithmic bytes) and the factorisation's effective rate (2/3 n^3 flops)."""
    out = {"assemble_gbs": 4.0 * n * n / (assemble_ms * 1e-3) / 1e9,
           "factor_tflops_effective": (2.0 / 3.0) * float(n) ** 3 / (factor_ms * 1e-3) / 1e12}
    pk = measured_peaks()
    if pk.get("hbm_gbs"):
        out["assemble_frac_of_hbm"] = out["assemble_gbs"] / pk["hbm_gbs"]
    return out


def bench_bem(args, G, torch, W, fp64=True):
    """BEM on a sphere: unit sphere from 5 icosahedral refinements (20,480 panels), freestream
    (1,0,0), 100,000 particles in the shell 1.02 < r < 1.5 (seed 3); RHS from the particles
    (points_affect_panels) plus freestream, influence matrix assembly, FP32/TF32 LU, FP64-
    residual refinement to 1e-10.  Reported for 2 unknowns per panel (n = 40,960) and the
    reference's default 3 (n = 61,440), after one untimed warm-up pass at each size."""
    out = {}
    x, i = G.generate_ovoid(args.bem_level, 2.0, 2.0, 2.0)
    px, ps, pr = W.shell_particles(100000, seed=3)
    src = G.Points(*(torch.from_numpy(a).cuda() for a in (px, ps, pr)))
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    for nunk in (2, 3):
        s = G.Surfaces(x, i, nunk=nunk)
        arr = s.device_arrays("cuda")
        n = s.npanels * nunk
        bem = G.BEM(n)
        res = {}
        for rep in range(2):
            e = [ev() for _ in range(10)]
            e[0].record()
            pu = torch.zeros(3, s.npanels, device="cuda")
            G.points_affect_panels(src, s, arrays=arr, pu=pu)
            rhs = torch.empty(n, device="cuda")
            st = G.influence.surface_struct(arr)
            fsd = (G.influence.ctypes.c_double * 3)(1.0, 0.0, 0.0)
            G.lib().o3g_panel_vels_to_rhs(s.npanels, nunk, fsd, *G.influence._rows(pu, 3),
                                          G.influence.ctypes.byref(st), rhs.data_ptr(), None)
            e[1].record()
            bem.assemble(arr, arr, nunk, True)
            e[2].record()
            bem.factor()
            e[3].record()
            xs = bem.solve(rhs, tol=1e-10, max_iter=30)
            e[4].record()
            torch.cuda.synchronize()
            res = {"n": n, "unknowns_per_panel": nunk, "rhs_ms": e[0].elapsed_time(e[1]),
                   "assemble_ms": e[1].elapsed_time(e[2]), "factor_ms": e[2].elapsed_time(e[3]),
                   "solve_ms": e[3].elapsed_time(e[4]), "refinements": bem.iters, "relres": bem.relres,
                   "total_ms": e[0].elapsed_time(e[4])}
            res.update(bem_rates(n, res["assemble_ms"], res["factor_ms"]))
            # the reference's own method on the same assembled matrix: GMRES, no factorisation
            e[5].record()
            xg = bem.solve(rhs, tol=1e-10, max_iter=300, method="gmres")
            e[6].record()
            torch.cuda.synchronize()
            res["gmres"] = {"solve_ms": e[5].elapsed_time(e[6]), "iterations": bem.iters, "relres": bem.relres,
                            "total_ms_with_rhs_and_assembly": e[0].elapsed_time(e[2]) + e[5].elapsed_time(e[6]),
                            "strengths_vs_lu_max_rel": float(((xg - xs).abs().max() / xs.abs().max()).item())}
            if nunk == 2 and rep == 1:
                res["many_rhs"] = bench_many_rhs(bem, rhs, torch, ev)
        if fp64 and nunk == 2:
            A = torch.empty((n, n), device="cuda")
            G.panels_on_panels_coeff(arr, arr, nunk, True, A)
            Ad = A.t().contiguous().double()
            del A
            bd = rhs.double()
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record()
            LU, piv = torch.linalg.lu_factor(Ad)
            xd = torch.linalg.lu_solve(LU, piv, bd[:, None])[:, 0]
            e1.record()
            torch.cuda.synchronize()
            res["fp64_lu_solve_ms"] = e0.elapsed_time(e1)
            res["fp64_lu_relres"] = float((torch.linalg.norm(bd - Ad @ xd) / torch.linalg.norm(bd)).item())
            res["strengths_vs_fp64_lu_max_rel"] = float(((xs.double() - xd).abs().max() / xd.abs().max()).item())
            res["speedup_vs_fp64_lu"] = res["fp64_lu_solve_ms"] / (res["factor_ms"] + res["solve_ms"])
            res["gmres"]["speedup_vs_fp64_lu"] = res["fp64_lu_solve_ms"] / res["gmres"]["solve_ms"]
            res["gmres"]["strengths_vs_fp64_lu_max_rel"] = float(((xg.double() - xd).abs().max() /
                                                                  xd.abs().max()).item())
            del Ad, LU, piv
        out["nunk%d" % nunk] = res
        del bem
        torch.cuda.empty_cache()
    return out


def bench_many_rhs(bem, rhs, torch, ev):
    """Several right-hand sides per matrix pass (o3g_bem_solve_many / _gmres_many) on the
    factorised sphere system: k = 1, 2, 4, 8 right-hand sides (the sphere's own RHS scaled
    and perturbed by seeded noise of 1e-3 of its size), each solved to 1e-10; time per
    right-hand side against one single-vector solve."""
    g = torch.Generator(device="cuda").manual_seed(5)
    out = {}
    single = {}
    for method, iters in (("lu", 30), ("gmres", 300)):
        e0, e1 = ev(), ev()
        e0.record()
        bem.solve(rhs, tol=1e-10, max_iter=iters, method=method)
        e1.record()
        torch.cuda.synchronize()
        single[method] = e0.elapsed_time(e1)
    for k in (1, 2, 4, 8):
        B = torch.stack([rhs * (1.0 + 0.1 * c) + 1e-3 * rhs.abs().max() *
                         torch.randn(rhs.shape[0], device="cuda", generator=g) for c in range(k)])
        row = {}
        for method, iters in (("lu", 30), ("gmres", 300)):
            e0, e1 = ev(), ev()
            e0.record()
            bem.solve_many(B, tol=1e-10, max_iter=iters, method=method)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            row[method] = {"ms": ms, "ms_per_rhs": ms / k, "per_rhs_vs_single": (ms / k) / single[method],
                           "max_relres": float(bem.relres_many.max()), "iterations": bem.iters_many.tolist()}
        out["k%d" % k] = row
    out["single_ms"] = single
    return out


def measured_peaks():
    """MEASURED_PEAKS.json (written beside this file by the measuring harness), or {}."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def bench_tc_gemm(G, torch, m=40448, n=40448, k=512, reps=5):
    """The LU's trailing update on its own: C -= A B (o3g_gemm_tf32_sub, tcgen05 kind::tf32)
    at the size of the first big update of the n = 40,960 factorisation (m = n = 40,448,
    k = 512, the outer panel).  Achieved TFLOP/s
    (2 m n k per call) against the TF32 tensor roof, taken as half the measured dense bf16
    rate (MEASURED_PEAKS.json bf16_tflops; TF32 runs at half the bf16 rate), and the HBM
    traffic the update cannot avoid (C read and written once, A and B read) against the
    measured copy bandwidth."""
    g = torch.Generator(device="cuda").manual_seed(11)
    A = torch.randn((k, m), device="cuda", generator=g)       # column-major m x k
    B = torch.randn((n, k), device="cuda", generator=g)       # column-major k x n
    C = torch.randn((n, m), device="cuda", generator=g)
    lib = G.lib()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    times = []
    for _ in range(reps + 1):
        e0, e1 = ev(), ev()
        e0.record()
        st = lib.o3g_gemm_tf32_sub(m, n, k, A.data_ptr(), m, B.data_ptr(), k, C.data_ptr(), m, None)
        e1.record()
        torch.cuda.synchronize()
        if st != 0:
            raise RuntimeError(lib.o3g_last_error().decode())
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times[1:])
    tflops = 2.0 * m * n * k / (ms * 1e-3) / 1e12
    gb = (2.0 * m * n + m * k + k * n) * 4 / 1e9
    pk = measured_peaks()
    out = {"m": m, "n": n, "k": k, "ms": ms, "tflops": tflops, "hbm_gb": gb, "gbs": gb / (ms * 1e-3),
           "note": "includes the K-major copy of A and the stream synchronisation of the entry point"}
    if pk.get("bf16_tflops"):
        out["tf32_roof_tflops"] = pk["bf16_tflops"] / 2.0
        out["frac_of_tf32_roof"] = tflops / out["tf32_roof_tflops"]
    if pk.get("hbm_gbs"):
        out["frac_of_hbm"] = out["gbs"] / pk["hbm_gbs"]
    return out


def bench_ring(args, G, torch, W):
    """Plain method, small: thin vortex ring, N = 16,384, Rosenhead-Moore core sigma 0.05:
    one vel+grad evaluation, then 10 Ralston RK2 steps of dt = 0.01 replayed from a CUDA graph."""
    x, s, r = W.vortex_ring(16384)
    X, S, R = (torch.from_numpy(a).cuda() for a in (x, s, r))
    E = torch.ones(16384, device="cuda")
    p = G.Points(X, S, R)
    for _ in range(3):
        p.zero_vels()
        G.points_affect_points(p, p, G.ResultsType(), G.ExecEnv("rm", "plain"))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    reps = 20
    for _ in range(reps):
        p.zero_vels()
        G.points_affect_points(p, p, G.ResultsType(), G.ExecEnv("rm", "plain"))
    e1.record()
    torch.cuda.synchronize()
    eval_ms = e0.elapsed_time(e1) / reps
    rk = G.Ralston(X.clone(), S.clone(), R, E, env=G.ExecEnv("rm", "plain"))
    rk.step(0.01, (0.0, 0.0, 0.0), 2)                  # direct step + capture
    torch.cuda.synchronize()
    e0.record()
    rk.step(0.01, (0.0, 0.0, 0.0), 10)
    e1.record()
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / 10
    # CPU baseline, timed in full: the oracle port (float pairs, double sums, OpenMP)
    import oracle as O
    nth = os.cpu_count() or 1
    t0 = time.perf_counter()
    O.points_affect_points(x, r, s, x, r, True, "rm", 1, nth)
    cpu_s = time.perf_counter() - t0
    return {"n": 16384, "core": "rm", "eval_ms": eval_ms,
            "eval_interactions_per_s": 16384.0 ** 2 / (eval_ms * 1e-3), "rk2_step_ms": step_ms,
            "rk2_steps": 10, "dt": 0.01, "graph": True,
            "cpu_baseline": {"eval_s": cpu_s, "interactions_per_s": 16384.0 ** 2 / cpu_s, "cores": nth,
                             "kind": "port", "sample": "the whole evaluation (16,384 x 16,384)"}}


def bench_batch(args, G, torch, W, flush):
    """Batching: 64 independent particle systems (sizes log-uniform in [1,024, 65,536], seed 4),
    each a Gaussian blob with 4,096 field points on a jittered grid; Gaussian core; velocity +
    gradient of every system in ONE persistent launch with the autotuned configuration (the
    first run tunes and caches it; reported separately), L2 flushed before every timed run.
    Compared with one points_affect_points call per (system, target set) and, for errors,
    with the FP64 path on the same GPU for every 8th system.  Then 100 Ralston steps of all
    systems replayed from a CUDA graph (each step: two batched evaluations)."""
    import ctypes
    from omega3d_gb300 import _lib as L
    from omega3d_gb300.metrics import linf_err, rel_err
    lib = L.lib()
    syst = W.batch_systems(64, seed=4)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    z = lambda *sh: torch.zeros(*sh, device="cuda")  # noqa: E731
    npart = sum(q[0].shape[1] for q in syst)
    nfld = sum(q[3].shape[1] for q in syst)
    pairs = float(sum(q[0].shape[1] * (q[0].shape[1] + q[3].shape[1]) for q in syst))
    out = {"systems": len(syst), "particles": npart, "field_points": nfld, "interactions_per_eval": pairs,
           "core": "gauss", "l2": "flushed before every timed evaluation"}
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def make():
        return [G.BatchSystem(t(x), t(s), t(r), z(3, x.shape[1]), z(9, x.shape[1]), t(f), z(3, f.shape[1]),
                              z(9, f.shape[1])) for x, s, r, f in syst]

    results = {}
    for core, prec in (("gauss", "compensated"), ("gauss", "plain"), ("rm", "compensated"), ("rm", "plain")):
        devs = make()
        b = G.Batch(devs, G.ExecEnv(core, prec))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run()
        torch.cuda.synchronize()
        first_s = time.perf_counter() - t0
        for _ in range(2):
            b.run()
        lib.o3g_set_timing(1)
        run_ms, kern_ms = [], []
        n0 = L.launch_count()
        reps = 5
        for _ in range(reps):
            flush.fill_(1)
            e0, e1 = ev(), ev()
            e0.record()
            b.run()
            e1.record()
            e1.synchronize()
            run_ms.append(e0.elapsed_time(e1))
            km = ctypes.c_float(0)
            L.check(lib.o3g_last_kernel_ms(ctypes.byref(km)), "o3g_last_kernel_ms")
            kern_ms.append(float(km.value))
        launches = (L.launch_count() - n0) / reps
        lib.o3g_set_timing(0)
        for d in devs:
            for a in (d.u, d.ug, d.fu, d.fug):
                a.zero_()
        b.run()
        torch.cuda.synchronize()
        results[(core, prec)] = devs
        rm, km = statistics.median(run_ms), statistics.median(kern_ms)
        out.setdefault(core, {})[prec] = {
            "value": pairs / (rm * 1e-3), "unit": UNIT, "run_ms": rm, "persistent_kernel_ms": km,
            "kernel_interactions_per_s": pairs / (km * 1e-3), "launches_per_run": launches,
            "first_run_s_incl_tuning": first_s, "config": b.config()}
        del b
    for core in ("gauss", "rm"):
        out[core]["compensated_over_plain"] = out[core]["plain"]["run_ms"] / out[core]["compensated"]["run_ms"]

    # one call per (system, target set): the unbatched way through the same library
    pts = [(G.Points(q.x, q.s, q.r), G.Points(q.f, None, None, inert=True)) for q in make()]
    for _ in range(2):
        for p, f in pts:
            p.zero_vels()
            f.zero_vels()
            G.points_affect_points(p, p, G.ResultsType(), G.ExecEnv("gauss", "compensated"))
            G.points_affect_points(p, f, G.ResultsType(), G.ExecEnv("gauss", "compensated"))
    loop_ms = []
    for _ in range(3):
        flush.fill_(1)
        e0, e1 = ev(), ev()
        e0.record()
        for p, f in pts:
            G.points_affect_points(p, p, G.ResultsType(), G.ExecEnv("gauss", "compensated"))
            G.points_affect_points(p, f, G.ResultsType(), G.ExecEnv("gauss", "compensated"))
        e1.record()
        e1.synchronize()
        loop_ms.append(e0.elapsed_time(e1))
    lm = statistics.median(loop_ms)
    out["per_system_calls"] = {"value": pairs / (lm * 1e-3), "unit": UNIT, "ms": lm, "calls": 2 * len(syst),
                               "core": "gauss", "precision": "compensated"}
    out["batched_over_per_system_calls"] = lm / out["gauss"]["compensated"]["run_ms"]
    del pts

    # errors against the FP64 path on the same GPU, every 8th system
    errs = {}
    for core, prec in results:
        mu = mg = 0.0
        su = sg = 0.0
        cnt = 0
        lu = lg = 0.0
        for k in range(0, len(syst), 8):
            x, s, r, f = syst[k]
            d = results[(core, prec)][k]
            src = G.Points(t(x.astype(np.float64)), t(s.astype(np.float64)), t(r.astype(np.float64)))
            for tx, tr, u, g in ((x, r, d.u, d.ug), (f, None, d.fu, d.fug)):
                tq = G.Points(t(tx.astype(np.float64)), None, None if tr is None else t(tr.astype(np.float64)),
                              inert=tr is None)
                G.points_affect_points(src, tq, G.ResultsType(), G.ExecEnv(core, "fp64"))
                u64, g64 = tq.u.cpu().numpy(), tq.ug.cpu().numpy()
                eu, eg = rel_err(u.cpu().numpy(), u64), rel_err(g.cpu().numpy(), g64)
                mu, mg = max(mu, eu[0]), max(mg, eg[0])
                su, sg, cnt = su + eu[1] ** 2, sg + eg[1] ** 2, cnt + 1
                lu = max(lu, linf_err(u.cpu().numpy(), u64))
                lg = max(lg, linf_err(g.cpu().numpy(), g64))
        errs["%s_%s" % (core, prec)] = {"u_max": mu, "u_rms": (su / cnt) ** 0.5, "grad_max": mg, "grad_rms": (sg / cnt) ** 0.5,
                      "u_linf": lu, "grad_linf": lg, "systems_checked": cnt // 2}
    out["errors_vs_fp64"] = errs
    # time step from the initial velocity gradients (dt * max |grad u| = 0.05): random-strength
    # blobs stretch their particles at a rate set by the largest gradient
    gmax = max(float(torch.linalg.norm(d.ug, dim=0).max().item()) for d in results[("gauss", "compensated")])
    dt = 0.05 / (gmax / (4 * np.pi))
    del results

    # 100 Ralston steps of all systems under a CUDA graph
    X = t(np.concatenate([q[0] for q in syst], axis=1))
    S = t(np.concatenate([q[1] for q in syst], axis=1))
    R = t(np.concatenate([q[2] for q in syst]))
    F = t(np.concatenate([q[3] for q in syst], axis=1))
    E = torch.ones(npart, device="cuda")
    rk = G.BatchRalston([q[0].shape[1] for q in syst], [q[3].shape[1] for q in syst], X, S, R, E, F,
                        G.ExecEnv("gauss", "compensated"))
    rk.step(dt, (0.0, 0.0, 0.0), 2)                 # direct step (sizes workspaces) + capture
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record(rk.stream)
    rk.step(dt, (0.0, 0.0, 0.0), 100)
    e1.record(rk.stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    out["rk2"] = {"steps": 100, "dt": dt, "core": "gauss", "precision": "compensated", "graph": True, "total_ms": ms,
                  "step_ms": ms / 100, "interactions_per_s": 2 * pairs * 100 / (ms * 1e-3),
                  "finite": bool(torch.isfinite(X).all().item())}
    del rk
    return out


def bench_coupled(args, G, torch, W):
    """Full coupled step at scale: unit sphere of 5,120 panels (4 icosahedral refinements,
    2 unknowns per panel), 1,048,576 particles uniform in the wake box x in [1, 6],
    |y|, |z| < 1.5 (seed 5, N(0, 1e-3^2) strengths, core radius 0.015), Rosenhead-Moore core,
    compensated FP32.  Each Ralston step (dt = 0.005, freestream (1, 0, 0)) solves the BEM at
    both stages for the stage's particles (RHS from 1,048,576 particles, the factorisation of
    the fixed body reused) and sums particle->particle and panel->particle vel+grad.
    Timed: the assembly + factorisation once, `--coupled-steps` steps, and the parts of one
    stage separately; the particle-particle sums' error against the FP64 path on the same
    GPU at 2,048 sampled particles (the panel sums are checked against FP64 by the tests)."""
    from omega3d_gb300.metrics import linf_err, rel_err
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    n = 1048576
    xs, idx = G.generate_ovoid(4, 2.0, 2.0, 2.0)
    surf = G.Surfaces(xs, idx, nunk=2)
    px, ps, pr = W.wake_particles(n, seed=5)
    X, S, R, E = t(px), t(ps), t(pr), torch.ones(n, device="cuda")
    env = G.ExecEnv("rm", "compensated")
    out = {"panels": surf.npanels, "unknowns": surf.npanels * 2, "particles": n, "core": "rm",
           "precision": "compensated", "dt": 0.005}
    rk = G.Ralston(X, S, R, E, env=env, use_graph=False)
    bem = G.BEM(surf.npanels * 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # clear_inner_layer after each move with ips = the nominal particle spacing of the wake box
    ips = float((5.0 * 3.0 * 3.0 / n) ** (1.0 / 3.0))
    rk.attach_body(surf, bem, ips=ips)
    torch.cuda.synchronize()
    out["assemble_factor_ms"] = (time.perf_counter() - t0) * 1e3
    out["ips"] = ips

    # the parts of one stage on the initial state
    arr = rk.body_arrays
    P = G.Points(X, S, R)
    e = [ev() for _ in range(4)]
    P.zero_vels()
    G.points_affect_points(P, P, G.ResultsType(), env)                  # warm-up
    torch.cuda.synchronize()
    pu = torch.zeros(3, surf.npanels, device="cuda")
    e[0].record()
    G.points_affect_panels(P, surf, env, arrays=arr, pu=pu)
    e[1].record()
    rng = np.random.default_rng(6)
    surf.set_sheet_strengths(rng.normal(size=surf.npanels).astype(np.float32) * 0.1,
                             rng.normal(size=surf.npanels).astype(np.float32) * 0.1)
    arr2 = surf.device_arrays("cuda")
    torch.cuda.synchronize()
    e[2].record()
    G.panels_affect_points(surf, P, G.ResultsType(), env, arrays=arr2)
    e[3].record()
    torch.cuda.synchronize()
    pairs = float(n) * n
    rhs_ms, pair_ms, pan_ms = e[0].elapsed_time(e[1]), None, e[2].elapsed_time(e[3])
    e0, e1 = ev(), ev()
    P.zero_vels()
    e0.record()
    G.points_affect_points(P, P, G.ResultsType(), env)
    e1.record()
    torch.cuda.synchronize()
    pair_ms = e0.elapsed_time(e1)
    out["stage_parts_ms"] = {"rhs_points_affect_panels": rhs_ms, "particle_particle": pair_ms,
                             "panel_particle": pan_ms}
    out["particle_particle_interactions_per_s"] = pairs / (pair_ms * 1e-3)
    out["panel_particle_pairs_per_s"] = float(surf.npanels) * n / (pan_ms * 1e-3)

    # error of the compensated particle-particle sums at sampled particles vs the FP64 path
    # (P holds the particle sums plus the panel sums of the last call: evaluate again)
    P.zero_vels()
    G.points_affect_points(P, P, G.ResultsType(), env)
    sub = np.linspace(0, n - 1, 2048).astype(np.int64)
    tq = G.Points(t(px[:, sub].astype(np.float64)), None, t(pr[sub].astype(np.float64)))
    G.points_affect_points(G.Points(t(px.astype(np.float64)), t(ps.astype(np.float64)), t(pr.astype(np.float64))),
                           tq, G.ResultsType(), G.ExecEnv("rm", "fp64"))
    u, g = P.u.cpu().numpy()[:, sub], P.ug.cpu().numpy()[:, sub]
    u64, g64 = tq.u.cpu().numpy(), tq.ug.cpu().numpy()
    out["particle_particle_errors_vs_fp64"] = {
        "u_max": rel_err(u, u64)[0], "u_rms": rel_err(u, u64)[1], "grad_max": rel_err(g, g64)[0],
        "u_linf": linf_err(u, u64), "grad_linf": linf_err(g, g64), "samples": 2048}
    del P, tq

    steps = args.coupled_steps
    e0, e1 = ev(), ev()
    torch.cuda.synchronize()
    e0.record(rk.stream)
    rk.step(0.005, (1.0, 0.0, 0.0), steps)
    e1.record(rk.stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    st = rk.body_stats()
    # one clear_inner_layer pass over all particles on its own (two run in every step)
    e0, e1 = ev(), ev()
    e0.record()
    pushed = G.clear_inner_layer(surf, G.Points(X, None, None, inert=True), ips=ips, arrays=arr)
    e1.record()
    torch.cuda.synchronize()
    out["clear_inner_layer_ms"] = e0.elapsed_time(e1)
    out["clear_inner_layer_point_panel_tests_per_s"] = float(n) * surf.npanels / (e0.elapsed_time(e1) * 1e-3)
    out["steps"] = steps
    out["step_ms"] = ms / steps
    out["interactions_per_step"] = 2 * (pairs + float(surf.npanels) * n * 2)
    # CPU baseline of the particle-particle sums, the step's dominant part: the oracle port
    # on a seeded 4,096-target subset against all 1,048,576 sources, scaled by rate
    import oracle as O
    nth = os.cpu_count() or 1
    sub = np.sort(np.random.default_rng(7).choice(n, 4096, replace=False))
    tx_, tr_ = np.ascontiguousarray(px[:, sub]), np.ascontiguousarray(pr[sub])
    t0 = time.perf_counter()
    O.points_affect_points(px, pr, ps, tx_, tr_, True, "rm", 1, nth)
    cpu_rate = 4096.0 * n / (time.perf_counter() - t0)
    out["cpu_baseline_particle_particle"] = {
        "interactions_per_s": cpu_rate, "stage_s_scaled": pairs / cpu_rate, "cores": nth, "kind": "port",
        "sample": "4,096 seeded targets x 1,048,576 sources (RM, float pairs, double sums)",
        "gpu_stage_speedup": (pairs / cpu_rate) / (pair_ms * 1e-3)}
    out["bem"] = st
    out["finite"] = bool(torch.isfinite(X).all().item())
    del rk, bem
    torch.cuda.empty_cache()
    return out


def bench_bem_cpu(W):
    """CPU baseline of the same BEM workload (20,480-panel sphere, 2 unknowns per panel,
    100,000 shell particles, freestream (1,0,0)) with the reference's own method.  It runs
    the oracle port of the reference's loops on all host cores: RHS (points_affect_panels +
    finalize + vels_to_rhs), assembly (panels_on_panels_coeff) and a restated Eigen GMRES
    (restart 30, diagonal preconditioner, float epsilon), all in FP32 like BEM<float,Int>."""
    import oracle as O
    nodes, idx = O.generate_ovoid(5, 2.0, 2.0, 2.0)
    x1, x2, nm, area = O.compute_bases(nodes, idx)
    geo = dict(nodes=nodes, idx=idx, area=area, x1=x1, x2=x2, norm=nm)
    px, ps, _ = W.shell_particles(100000, seed=3)
    t0 = time.perf_counter()
    pu = O.points_affect_panels(px, ps, nodes, idx, area, "rm", 0)
    O.finalize_vels(pu, None, (1.0, 0.0, 0.0))
    b = O.vels_to_rhs_panels(pu, x1, x2, nm, 2)
    t1 = time.perf_counter()
    C = O.panels_on_panels_coeff(geo, geo, 2, True, "rm", 0)
    t2 = time.perf_counter()
    _, it, rel = O.gmres_restarted(C.T, b)
    t3 = time.perf_counter()
    del C
    # FP64 LU (numpy / LAPACK on all host cores) of the 10,240-unknown system of the
    # 4-level sphere, a bounded sample: the full 40,960-unknown factorisation would take
    # minutes; its time scales as n^3
    n4, i4 = O.generate_ovoid(4, 2.0, 2.0, 2.0)
    a1, a2, an, aa = O.compute_bases(n4, i4)
    C4 = O.panels_on_panels_coeff(dict(nodes=n4, idx=i4, area=aa, x1=a1, x2=a2, norm=an),
                                  dict(nodes=n4, idx=i4, area=aa, x1=a1, x2=a2, norm=an), 2, True, "rm", 0)
    A4 = np.ascontiguousarray(C4.T, dtype=np.float64)
    b4 = np.zeros(A4.shape[0])
    b4[0::2], b4[1::2] = -a1[0], -a2[0]
    t4 = time.perf_counter()
    np.linalg.solve(A4, b4)
    lu4 = time.perf_counter() - t4
    n = int(b.shape[0])
    return {"n": n, "rhs_s": t1 - t0, "assemble_s": t2 - t1, "gmres_s": t3 - t2,
            "gmres_iterations": it, "gmres_relres": rel, "total_s": t3 - t0, "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": "the whole workload: oracle loops (OpenMP) + restated Eigen GMRES in numpy FP32",
            "fp64_lu": {"n": int(A4.shape[0]), "solve_s": lu4, "scaled_to_n_s": lu4 * (n / A4.shape[0]) ** 3,
                        "sample": "numpy FP64 LU solve of the 4-level sphere's system, scaled by n^3 to n"}}


def cpu_splitmerge(x, s, r, e):
    """The oracle port of Split.h / Merge.h on the host, single thread (the reference's loops
    are sequential), run twice: with the restated nanoflann kd-tree, the reference's own
    search structure, timed as the CPU baseline; and with the cell list, which takes
    equal-distance neighbours in increasing index like the kernels, for the bit-for-bit
    check.  Returns {order: (split result, split ms, merge result, merge ms)}."""
    import oracle as O
    res = {}
    for order in ("kdtree", "index"):
        t0 = time.perf_counter()
        sp = O.split_elongated(x, s, r, e, 0, 1.5, 1.2, tie_order=order)
        t_sp = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        mg = O.merge_close_particles(x, s, r, 1.5, 0.2, False, tie_order=order)
        t_mg = (time.perf_counter() - t0) * 1e3
        res[order] = (sp, t_sp, mg, t_mg)
    return res


def bench_splitmerge(args, G, torch, W, reps=3, k=100):
    """Particle split (Split.h:44-270) and merge (Merge.h:45-218) of 1,000,000 particles on
    a jittered lattice (19 % elongated past the split threshold, 9 % with a neighbour within
    half a separation).  Each call is timed end to end (both wait for their result) on fresh
    device copies; the oracle port of the reference's sequential loops runs on the host for
    the CPU figure and to confirm the device results bit for bit (cpu_splitmerge)."""
    x, s, r, e = W.lattice_particles(k=k, seed=41)
    n = x.shape[1]
    dev = torch.device("cuda", torch.cuda.current_device())
    X, S, R, E = (torch.from_numpy(a).to(dev) for a in (x, s, r, e))
    out = {"particles": n, "overlap": 1.5, "split_threshold": 1.2, "merge_threshold": 0.2}

    def timed(fn):
        ts = []
        res = None
        for it in range(reps + 1):
            args_ = (X.clone(), S.clone(), R.clone(), E.clone())
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = fn(*args_)
            torch.cuda.synchronize()
            if it > 0:
                ts.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(ts), res

    sp_ms, sp = timed(lambda a, b, c, d: G.split_elongated(a, b, c, d, "gaussian", 1.5, 1.2))
    mg_ms, mg = timed(lambda a, b, c, d: G.merge_close_particles(a, b, c, 1.5, 0.2, False))
    cpu = cpu_splitmerge(x, s, r, e)
    osp, cell_sp, omg, cell_mg = cpu["index"]
    _, cpu_sp, _, cpu_mg = cpu["kdtree"]

    def same(dev_arrs, host_arrs):
        return all(np.array_equal(a.cpu().numpy().view(np.uint32), np.ascontiguousarray(b).view(np.uint32))
                   for a, b in zip(dev_arrs, host_arrs))

    kd_sp, kd_mg = cpu["kdtree"][0], cpu["kdtree"][2]
    out["split"] = {"ms": sp_ms, "particles_per_s": n / (sp_ms * 1e-3), "nsplit": sp[4],
                    "cpu_port_ms": cpu_sp, "speedup_vs_cpu_port": cpu_sp / sp_ms, "cpu_port_cell_list_ms": cell_sp,
                    "bit_identical_to_port": bool(sp[4] == osp[4] and same(sp[:4], osp[:4])),
                    "port_kdtree_equals_cell_list": bool(kd_sp[4] == osp[4] and all(
                        np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(kd_sp[:4], osp[:4])))}
    out["merge"] = {"ms": mg_ms, "particles_per_s": n / (mg_ms * 1e-3), "nremoved": mg[3],
                    "cpu_port_ms": cpu_mg, "speedup_vs_cpu_port": cpu_mg / mg_ms, "cpu_port_cell_list_ms": cell_mg,
                    "bit_identical_to_port": bool(mg[3] == omg[3] and same(mg[:3], omg[:3])),
                    "port_kdtree_equals_cell_list": bool(kd_mg[3] == omg[3] and all(
                        np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(kd_mg[:3], omg[:3])))}
    out["cpu_port"] = {"cores": 1, "kind": "port",
                       "sample": "the whole 1,000,000-particle operator, single thread (the reference's loops are "
                                 "sequential), neighbours found with the restated nanoflann kd-tree the reference "
                                 "uses; cpu_port_cell_list_ms is the same port with the cell list"}
    return out


def guarded(fn):
    """Runs one secondary section of the line.  An exception there is reported in the line as
    that section's {"error": ...} instead of losing the headline."""
    try:
        return fn()
    except Exception as ex:
        return {"error": "%s: %s" % (type(ex).__name__, str(ex)[:500])}


def bem_section(args, G, torch, W, rank):
    bem = bench_bem(args, G, torch, W, fp64=not args.skip_bem_fp64)
    bem["tc_gemm_update"] = guarded(lambda: bench_tc_gemm(G, torch))
    if rank == 0:
        bem["cpu_baseline_nunk2"] = cpu = bench_bem_cpu(W)
        g = bem["nunk2"]["gmres"]["total_ms_with_rhs_and_assembly"] * 1e-3
        cpu["gpu_gmres_speedup"] = cpu["total_s"] / g
    return bem


def run_ours(args):
    import torch
    import torch.distributed as dist

    import omega3d_gb300 as G
    from omega3d_gb300 import _lib as L
    from omega3d_gb300 import workloads as W
    from omega3d_gb300.metrics import linf_err, rel_err

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
        # replicas: the flagship cloud section only; the other workloads are single-GPU
        # reports and would hold every GPU (and the shared host cores) for minutes
        args.skip_bem = args.skip_ring = args.skip_batch = args.skip_splitmerge = True
        args.coupled_steps = 0
    lib = L.lib()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    if args.only:
        # one workload section alone (for profiling it); prints that section's results only
        fn = {"bem": lambda: bench_bem(args, G, torch, W, fp64=not args.skip_bem_fp64),
              "ring": lambda: bench_ring(args, G, torch, W),
              "batch": lambda: bench_batch(args, G, torch, W, flush),
              "coupled": lambda: bench_coupled(args, G, torch, W),
              "splitmerge": lambda: bench_splitmerge(args, G, torch, W),
              "gemm": lambda: {"%dx%dx%d" % mnk: bench_tc_gemm(G, torch, *mnk)
                               for mnk in ((8192, 8192, 512), (16384, 16384, 512), (40448, 40448, 512),
                                           (40448, 384, 128))}}[args.only]
        res = fn()
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"section": args.only, "result": res}))
        return

    x, s, r = W.gaussian_cloud(args.n, seed=2)
    X, S, R = (torch.from_numpy(a).to(dev) for a in (x, s, r))
    stream = torch.cuda.current_stream()

    nsm = int(torch.cuda.get_device_properties(dev).multi_processor_count)
    tfl, ms = ctypes.c_double(0), ctypes.c_float(0)
    L.check(lib.o3g_fp32_peak_probe(20000, stream.cuda_stream, ctypes.byref(tfl),
                                    ctypes.byref(ms)), "o3g_fp32_peak_probe")
    fp32_peak = float(tfl.value)

    fl_pair = lib.o3g_flops_per_pair(L.CORES[args.core], 1, 1)
    pairs = float(args.n) * args.n
    ref_flops = pairs * fl_pair + 12.0 * args.n

    def one(prec, p=None, core=None):
        p = p or G.Points(X, S, R)
        p.zero_vels()
        G.points_affect_points(p, p, G.ResultsType(), G.ExecEnv(core or args.core, prec))
        return p

    def timed(prec, steps, warmup, core=None):
        p = G.Points(X, S, R)
        for _ in range(warmup):
            one(prec, p, core)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        lib.o3g_set_timing(1)
        n0 = L.launch_count()
        step_ms, kern_ms = [], []
        t0 = time.perf_counter()
        for _ in range(steps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one(prec, p, core)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            km = ctypes.c_float(0)
            L.check(lib.o3g_last_kernel_ms(ctypes.byref(km)), "o3g_last_kernel_ms")
            kern_ms.append(float(km.value))
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        wall = time.perf_counter() - t0
        launches = L.launch_count() - n0
        lib.o3g_set_timing(0)
        return p, step_ms, kern_ms, wall, launches

    clocks = ClockSampler(local)
    clocks.start()
    pc, comp_ms, comp_kms, comp_wall, comp_launches = timed("compensated", args.steps, args.warmup)
    pp, plain_ms, plain_kms, _, _ = timed("plain", args.steps, args.warmup)
    # the Rosenhead-Moore core (no distance branches) on the same cloud, for the FP32 roofline
    rm = {}
    for prec in ("plain", "compensated"):
        _, rms, rkms, _, _ = timed(prec, args.steps, args.warmup, core="rm")
        fl_rm = lib.o3g_flops_per_pair(L.CORES["rm"], 1, 1)
        kms = statistics.median(rkms)
        rm[prec] = {"value": pairs / (statistics.median(rms) * 1e-3), "unit": UNIT, "kernel_ms": kms,
                    "roofline_frac": (pairs * fl_rm + 12.0 * args.n) / (kms * 1e-3) / 1e12 / fp32_peak}
    # the accurate mode (double-single pair terms, compensated sums) on the same cloud
    pa, acc_ms, acc_kms, _, _ = timed("accurate", args.steps, args.warmup)
    clk = clocks.stop()

    # e2e through the C-ABI with pinned host buffers: H2D + sums + D2H every step
    pinned = [torch.from_numpy(a).pin_memory() for a in (x, s, r)]
    pinned += [torch.zeros(3, args.n).pin_memory(), torch.zeros(9, args.n).pin_memory()]
    hp = G.Points(pinned[0].numpy(), pinned[1].numpy(), pinned[2].numpy(), u=pinned[3].numpy(),
                  ug=pinned[4].numpy())
    for _ in range(max(1, args.warmup)):
        hp.zero_vels()
        G.points_affect_points(hp, hp, G.ResultsType(), G.ExecEnv(args.core, "compensated"))
    e2e_s = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        hp.zero_vels()
        t0 = time.perf_counter()
        G.points_affect_points(hp, hp, G.ResultsType(), G.ExecEnv(args.core, "compensated"))
        e2e_s.append(time.perf_counter() - t0)
    h2d = 7 * 4 * args.n + 12 * 4 * args.n     # 7 source arrays + the 12 output arrays staged in
    d2h = 12 * 4 * args.n

    # FP64 comparator on the same GPU (subset of targets) and the errors of every path
    nsub = min(args.n, 16384)
    sub = torch.linspace(0, args.n - 1, nsub, device=dev).long()
    fp64 = None
    if not args.skip_fp64:
        Xd, Sd, Rd = X.double(), S.double(), R.double()
        tq = G.Points(Xd[:, sub].contiguous(), None, Rd[sub].contiguous())
        src = G.Points(Xd, Sd, Rd)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        G.points_affect_points(src, tq, G.ResultsType(), G.ExecEnv(args.core, "fp64"))
        e1.record(stream)
        e1.synchronize()
        fp64_rate = float(nsub) * args.n / (e0.elapsed_time(e1) * 1e-3)
        u64, g64 = tq.u.cpu().numpy(), tq.ug.cpu().numpy()
        subn = sub.cpu().numpy()
        errs = {}
        for name, p in (("compensated", pc), ("plain", pp), ("accurate", pa)):
            eu = rel_err(p.u.cpu().numpy()[:, subn], u64)
            eg = rel_err(p.ug.cpu().numpy()[:, subn], g64)
            errs[name] = {"u_max": eu[0], "u_rms": eu[1], "grad_max": eg[0], "grad_rms": eg[1],
                          "u_linf": linf_err(p.u.cpu().numpy()[:, subn], u64),
                          "grad_linf": linf_err(p.ug.cpu().numpy()[:, subn], g64)}
        fp64 = {"value": fp64_rate, "unit": UNIT, "targets": nsub, "errors_vs_fp64": errs}

    comp_step = statistics.median(comp_ms)
    plain_step = statistics.median(plain_ms)
    comp_k = statistics.median(comp_kms)
    plain_k = statistics.median(plain_kms)
    local_rate = pairs / (comp_step * 1e-3)

    # whole-job numbers: max time over ranks, interactions summed
    value, step_max = whole_job(comp_step, pairs, world, dist if world > 1 else None, dev)

    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        try:
            tr = json.load(open(tpath)).get("k_pair_gauss_compensated")
            if tr and tr.get("n") and tr.get("bytes"):
                traffic = tr["bytes"] * (args.n / tr["n"]) ** 2 if tr.get("scales") == "n^2" else tr["bytes"]
        except Exception:
            traffic = None

    bem = None
    if not args.skip_bem:
        bem = guarded(lambda: bem_section(args, G, torch, W, rank))
    ring = None
    if not args.skip_ring:
        ring = guarded(lambda: bench_ring(args, G, torch, W))
    batch = None
    if not args.skip_batch:
        batch = guarded(lambda: bench_batch(args, G, torch, W, flush))
    coupled = None
    if args.coupled_steps > 0:
        coupled = guarded(lambda: bench_coupled(args, G, torch, W))
    splitmerge = None
    if not args.skip_splitmerge:
        splitmerge = guarded(lambda: bench_splitmerge(args, G, torch, W))

    if rank == 0:
        cpu_v, cpu_cores, cpu_sample, _ = cpu_reference(args)
        achieved = ref_flops / (comp_k * 1e-3) / 1e12
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(args),
            "path": "compensated FP32 (two-sum accumulators, Newton-refined rsqrt)",
            "error_vs_fp64": fp64["errors_vs_fp64"]["compensated"] if fp64 else None,
            "e2e": {"value": world * pairs / statistics.median(e2e_s), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "path": "o3g_points_affect_points, O3G_MEM_HOST, pinned buffers"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak, "traffic": traffic,
                         "kernel": "k_pair<GAUSS, COMPENSATED, grads>",
                         "flops_per_interaction": fl_pair,
                         "peak_source": "measured in this run: o3g_fp32_peak_probe FMA chains (no FP32 figure in "
                                        "MEASURED_PEAKS.json)",
                         "kernel_ms": comp_k},
            "plain": {"value": world * pairs / (plain_step * 1e-3), "unit": UNIT, "kernel_ms": plain_k,
                      "roofline_frac": ref_flops / (plain_k * 1e-3) / 1e12 / fp32_peak,
                      "error_vs_fp64": fp64["errors_vs_fp64"]["plain"] if fp64 else None},
            "compensated_over_plain": plain_step / comp_step,
            "accurate": {"value": world * pairs / (statistics.median(acc_ms) * 1e-3), "unit": UNIT,
                         "kernel_ms": statistics.median(acc_kms),
                         "over_plain": plain_step / statistics.median(acc_ms),
                         "path": "double-single pair terms (exact separation, d^2, core, cross product), "
                                 "velocity in double-single running sums, two-sum folds",
                         "error_vs_fp64": fp64["errors_vs_fp64"]["accurate"] if fp64 else None},
            "rm_core_same_cloud": rm,
            "fp64_same_gpu": fp64 and {"value": fp64["value"], "unit": UNIT, "targets": fp64["targets"],
                                       "compensated_speedup": local_rate / fp64["value"]},
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cpu_cores, "kind": "port", "sample": cpu_sample},
            "bem_solve": bem, "ring_rk2": ring, "batch": batch, "coupled": coupled, "split_merge": splitmerge,
            "clocks": clk, "gpu_launches": comp_launches, "num_sms": nsm,
            "wall_s_timed_region": comp_wall,
        }
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
