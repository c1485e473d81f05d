"""Reference-shaped call surface over the C-ABI: Points / ResultsType / ExecEnv /
points_affect_points, mirroring Omega3D's Influence.h:67 (points_affect_points),
Points.h (the SoA particle container) and ExecEnv.h / ResultsType.h.

Arrays are either numpy arrays (host memory: the C-ABI stages them through the GPU
inside the call) or torch CUDA tensors (device memory: the call is asynchronous on
the given stream).  Positions/strengths/velocities are [3, n], gradients [9, n] in
the reference order (Kernels.h:184-192), radii/elongations [n]; all float32 (or all
float64 for the double entry point).
"""
import ctypes

import numpy as np

from . import _lib as L

try:  # torch is only needed for device-resident arrays
    import torch
except Exception:  # pragma: no cover
    torch = None


class ResultsType:
    """ResultsType.h: which results a target wants."""
    velonly = "velonly"
    velandgrad = "velandgrad"

    def __init__(self, kind="velandgrad"):
        if kind not in (self.velonly, self.velandgrad):
            raise ValueError("ResultsType must be 'velonly' or 'velandgrad'")
        self.kind = kind

    def compute_grad(self):
        return self.kind == self.velandgrad


class ExecEnv:
    """ExecEnv.h counterpart: core function, pair-sum precision and CUDA stream."""

    def __init__(self, core="rm", precision="plain", stream=None):
        if core not in L.CORES:
            raise ValueError("unknown core %r" % (core,))
        if precision not in L.PRECS:
            raise ValueError("unknown precision %r" % (precision,))
        self.core = core
        self.precision = precision
        self.stream = stream

    def stream_handle(self, on_device):
        if self.stream is None:
            if on_device and torch is not None:
                return torch.cuda.current_stream().cuda_stream
            return 0
        if torch is not None and isinstance(self.stream, torch.cuda.Stream):
            return self.stream.cuda_stream
        return int(self.stream)


def _is_dev(a):
    return torch is not None and isinstance(a, torch.Tensor) and a.is_cuda


def _dtype_ok(a, dt):
    if _is_dev(a):
        return a.dtype == (torch.float32 if dt == np.float32 else torch.float64) and a.is_contiguous()
    return isinstance(a, np.ndarray) and a.dtype == dt and a.flags["C_CONTIGUOUS"]


def _base(a):
    return a.data_ptr() if _is_dev(a) else a.ctypes.data


def _rows(a, k):
    """Pointers to the k component rows of a C-contiguous [k, n] array."""
    n = a.shape[1]
    item = a.element_size() if _is_dev(a) else a.itemsize
    b = _base(a)
    return [b + i * n * item for i in range(k)]


class _DeviceArray:
    """A device buffer described by __cuda_array_interface__ (torch wraps it without a copy)."""

    def __init__(self, ptr, shape, strides, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "strides": tuple(strides), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 2}


def device_matrix_view(base, ld, nrows, ncols=None):
    """The column-major FP32 matrix at device address `base` (leading dimension ld), e.g. the
    BEM handle's (BEM.matrix()), as a torch tensor M of shape (ncols, nrows) whose row j is
    column j of the matrix.  A view of that memory: no copy, no allocation."""
    if torch is None:
        raise RuntimeError("device_matrix_view needs torch")
    ncols = nrows if ncols is None else ncols
    return torch.as_tensor(_DeviceArray(base, (ncols, nrows), (4 * ld, 4), "<f4"), device="cuda")


class Points:
    """Points<S> (Points.h:50-140): positions x[3,n], strengths s[3,n], core radii r[n],
    velocities u[3,n] and optional gradients ug[9,n].  `inert` marks field points
    (elem_t inert, Omega3D.h:33): they have no radius and no strength."""

    def __init__(self, x, s=None, r=None, inert=False, grads=True, u=None, ug=None):
        self.x = x
        self.s = s
        self.r = r
        self.inert = inert
        n = x.shape[1]
        dev = _is_dev(x)
        dt = x.dtype
        if u is None:
            u = torch.zeros((3, n), dtype=dt, device=x.device) if dev else np.zeros((3, n), dt)
        if ug is None and grads:
            ug = torch.zeros((9, n), dtype=dt, device=x.device) if dev else np.zeros((9, n), dt)
        self.u = u
        self.ug = ug

    @property
    def n(self):
        return self.x.shape[1]

    def zero_vels(self):
        """ElementBase.h:174-184 / Points.h:255-262."""
        for a in (self.u, self.ug):
            if a is not None:
                a[...] = 0

    def finalize_vels(self, fs=(0.0, 0.0, 0.0)):
        """u = fs + u/(4 pi); ug *= 1/(4 pi)  (ElementBase.h:187-193, Points.h:265-277)."""
        fac = 0.25 / np.pi
        for d in range(3):
            self.u[d] = fs[d] + self.u[d] * fac
        if self.ug is not None:
            self.ug *= np.float32(fac) if self.ug.dtype in (np.float32,) else fac


def points_affect_points(src, targ, restype=None, env=None):
    """Influence.h:67: accumulate (+=) the velocity (and gradients) induced by the vortex
    particles `src` at the points `targ`.  No 1/4pi factor (see Points.finalize_vels)."""
    restype = restype or ResultsType()
    env = env or ExecEnv()
    if src.inert:
        raise ValueError("inert points cannot be sources")
    grads = restype.compute_grad()
    if grads and targ.ug is None:
        raise ValueError("targets have no velocity-gradient arrays")
    dt = np.float64 if (src.x.dtype in (np.float64,) or (_is_dev(src.x) and src.x.dtype == torch.float64)) \
        else np.float32
    arrays = [src.x, src.s, src.r, targ.x, targ.u] + ([targ.ug] if grads else []) + \
             ([targ.r] if not targ.inert else [])
    on_dev = _is_dev(src.x)
    for a in arrays:
        if _is_dev(a) != on_dev:
            raise ValueError("all arrays must live in the same memory (numpy host or torch CUDA)")
        if not _dtype_ok(a, dt):
            raise ValueError("arrays must be C-contiguous %s" % np.dtype(dt).name)
    sxp = _rows(src.x, 3)
    ssp = _rows(src.s, 3)
    txp = _rows(targ.x, 3)
    tup = _rows(targ.u, 3)
    tug = None
    if grads:
        tug = (ctypes.c_void_p * 9)(*_rows(targ.ug, 9))
    tr = None if targ.inert else _base(targ.r)
    mem = L.MEM_DEVICE if on_dev else L.MEM_HOST
    stream = env.stream_handle(on_dev)
    lib = L.lib()
    if dt == np.float64:
        st = lib.o3g_points_affect_points_d(L.CORES[env.core], mem, src.n, *sxp, _base(src.r), *ssp,
                                            targ.n, *txp, tr, *tup, tug, stream)
        L.check(st, "o3g_points_affect_points_d")
    else:
        st = lib.o3g_points_affect_points(L.CORES[env.core], L.PRECS[env.precision], mem, src.n, *sxp,
                                          _base(src.r), *ssp, targ.n, *txp, tr, *tup, tug, stream)
        L.check(st, "o3g_points_affect_points")


class InfluenceVisitor:
    """Influence.h:1251-1261: dispatch on (source kind, target kind)."""

    def __init__(self, restype=None, env=None):
        self.restype = restype or ResultsType()
        self.env = env or ExecEnv()

    def __call__(self, src, targ):
        if isinstance(src, Points) and isinstance(targ, Points):
            return points_affect_points(src, targ, self.restype, self.env)
        if isinstance(src, Surfaces) and isinstance(targ, Points):
            return panels_affect_points(src, targ, self.restype, self.env)
        if isinstance(src, Points) and isinstance(targ, Surfaces):
            return points_affect_panels(src, targ, self.env)
        if isinstance(src, Surfaces) and isinstance(targ, Surfaces):
            return panels_affect_panels(src, targ, self.env)
        raise NotImplementedError("pairing %s -> %s" % (type(src).__name__, type(targ).__name__))


# ------------------------------------------------------------------------------------
# surfaces

def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def generate_ovoid(levels, rx=1.0, ry=1.0, rz=1.0):
    """GeomHelper.cpp:41-91: icosahedral sphere of radius 0.5 refined `levels` times and
    scaled by (rx, ry, rz).  Returns nodes x[3, nn] (float32) and idx[3*np] (uint32)."""
    lib = L.lib()
    nn, np_ = ctypes.c_int32(), ctypes.c_int32()
    L.check(lib.o3g_ovoid_size(levels, ctypes.byref(nn), ctypes.byref(np_)), "o3g_ovoid_size")
    x = np.zeros((3, nn.value), np.float32)
    idx = np.zeros(3 * np_.value, np.uint32)
    L.check(lib.o3g_generate_ovoid(levels, rx, ry, rz, *_rows(x, 3), idx.ctypes.data), "o3g_generate_ovoid")
    return x, idx


class Surfaces:
    """Surfaces<S> (Surfaces.h:60-225): nodes x[3,nn], panel node indices idx[3*np], and
    per panel the basis x1/x2/norm [3,np], area [np], vortex-sheet strengths ps[3,np] (x1,
    x2, source), absolute strengths ts[3,np] and panel-centre velocities pu[3,np].  Built
    on the host (numpy); `to(device)` returns torch copies of the arrays for device calls.
    nunk = 3 when the source strength is unknown (the reference's default,
    Surfaces.h:71), 2 for tangential vortex sheets only."""

    def __init__(self, x, idx, nunk=3):
        self.x = _f32(x)
        self.idx = np.ascontiguousarray(idx, np.uint32)
        self.nunk = nunk
        nn, np_ = self.x.shape[1], self.idx.shape[0] // 3
        self.x1 = np.zeros((3, np_), np.float32)
        self.x2 = np.zeros((3, np_), np.float32)
        self.norm = np.zeros((3, np_), np.float32)
        self.area = np.zeros(np_, np.float32)
        L.check(L.lib().o3g_compute_bases(nn, *_rows(self.x, 3), np_, self.idx.ctypes.data, *_rows(self.x1, 3),
                                          *_rows(self.x2, 3), *_rows(self.norm, 3), self.area.ctypes.data),
                "o3g_compute_bases")
        self.ps = np.zeros((3, np_), np.float32)
        self.ts = np.zeros((3, np_), np.float32)
        self.pu = np.zeros((3, np_), np.float32)

    @property
    def npanels(self):
        return self.area.shape[0]

    @property
    def nnodes(self):
        return self.x.shape[1]

    def set_sheet_strengths(self, ps0, ps1, src=None):
        """Surfaces::set_str (Surfaces.h:267-306) without the BEM offsets."""
        self.ps[0], self.ps[1] = ps0, ps1
        if src is not None:
            self.ps[2] = src
        L.check(L.lib().o3g_sheet_to_panel_strength(self.npanels, self.ps[0].ctypes.data, self.ps[1].ctypes.data,
                                                    *_rows(self.x1, 3), *_rows(self.x2, 3), self.area.ctypes.data,
                                                    *_rows(self.ts, 3)), "o3g_sheet_to_panel_strength")

    def device_arrays(self, device):
        import torch
        keys = ("x", "idx", "area", "x1", "x2", "norm", "ps", "ts", "pu")
        out = {}
        for k in keys:
            a = getattr(self, k)
            t = torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(device)
            out[k] = t
        return out


def surface_struct(arr, nunk=3):
    """o3g_surface_t over a dict of arrays (numpy or torch, as returned by device_arrays)."""
    x, x1, x2, nm = arr["x"], arr["x1"], arr["x2"], arr["norm"]
    s = L.Surface()
    s.nn = x.shape[1]
    s.x, s.y, s.z = _rows(x, 3)
    s.np = arr["area"].shape[0]
    s.idx = _base(arr["idx"])
    s.area = _base(arr["area"])
    s.x1x, s.x1y, s.x1z = _rows(x1, 3)
    s.x2x, s.x2y, s.x2z = _rows(x2, 3)
    s.nx, s.ny, s.nz = _rows(nm, 3)
    return s


def _panel_prec(env):
    if env.precision not in ("plain", "compensated"):
        raise ValueError("panel influence runs in 'plain' or 'compensated' precision")
    return L.PRECS[env.precision]


def panels_affect_points(src, targ, restype=None, env=None, maxlev=3, arrays=None):
    """Influence.h:557: accumulate the velocity (and gradients) of the panels of `src` at the
    points of `targ`.  `arrays` (from src.device_arrays) selects device memory; otherwise
    the host arrays of `src` are used and targ must be numpy."""
    restype = restype or ResultsType()
    env = env or ExecEnv()
    grads = restype.compute_grad()
    a = arrays or {"x": src.x, "idx": src.idx, "area": src.area, "ts": src.ts, "ps": src.ps}
    on_dev = _is_dev(a["x"])
    if _is_dev(targ.x) != on_dev:
        raise ValueError("surface and targets must live in the same memory")
    tug = (ctypes.c_void_p * 9)(*_rows(targ.ug, 9)) if grads else None
    sss = _rows(a["ps"], 3)[2] if src.nunk == 3 else None
    st = L.lib().o3g_panels_affect_points(_panel_prec(env), L.MEM_DEVICE if on_dev else L.MEM_HOST, maxlev,
                                          a["x"].shape[1],
                                          *_rows(a["x"], 3), a["area"].shape[0], _base(a["idx"]), _base(a["area"]),
                                          *_rows(a["ts"], 3), sss, targ.n, *_rows(targ.x, 3), *_rows(targ.u, 3),
                                          tug, env.stream_handle(on_dev))
    L.check(st, "o3g_panels_affect_points")


def panels_affect_panels(src, targ, env=None, maxlev=3, src_arrays=None, targ_arrays=None, pu=None):
    """Influence.h:1223: the velocity of the panels of `src` at the collocation points of the
    panels of `targ` (centroids 0.0001 along the normal), WRITTEN into the target's panel
    velocities (targ.pu, or the [3, np] tensor `pu` with device arrays), as the reference
    copies them.  Device arrays when src_arrays / targ_arrays are given."""
    env = env or ExecEnv()
    a = src_arrays or {"x": src.x, "idx": src.idx, "area": src.area, "ts": src.ts, "ps": src.ps}
    t = targ_arrays or {"x": targ.x, "idx": targ.idx, "norm": targ.norm}
    on_dev = _is_dev(a["x"])
    if _is_dev(t["x"]) != on_dev:
        raise ValueError("source and target surfaces must live in the same memory")
    out = pu if pu is not None else targ.pu
    if _is_dev(out) != on_dev:
        raise ValueError("the velocity array must live with the surfaces")
    sss = _rows(a["ps"], 3)[2] if src.nunk == 3 else None
    st = L.lib().o3g_panels_affect_panels(_panel_prec(env), L.MEM_DEVICE if on_dev else L.MEM_HOST, maxlev,
                                          a["x"].shape[1], *_rows(a["x"], 3), a["area"].shape[0], _base(a["idx"]),
                                          _base(a["area"]), *_rows(a["ts"], 3), sss,
                                          t["x"].shape[1], *_rows(t["x"], 3), targ.npanels, _base(t["idx"]),
                                          *_rows(t["norm"], 3), *_rows(out, 3), env.stream_handle(on_dev))
    L.check(st, "o3g_panels_affect_panels")
    return out


def points_affect_panels(src, targ, env=None, maxlev=3, arrays=None, pu=None):
    """Influence.h:1107: subtract the panel-averaged velocity of the particles `src` from the
    panel velocities of `targ` (pu, or targ.pu on the host)."""
    env = env or ExecEnv()
    a = arrays or {"x": targ.x, "idx": targ.idx, "area": targ.area}
    pu = targ.pu if pu is None else pu
    on_dev = _is_dev(a["x"])
    st = L.lib().o3g_points_affect_panels(_panel_prec(env), L.MEM_DEVICE if on_dev else L.MEM_HOST, maxlev, src.n,
                                          *_rows(src.x, 3),
                                          *_rows(src.s, 3), a["x"].shape[1], *_rows(a["x"], 3), a["area"].shape[0],
                                          _base(a["idx"]), _base(a["area"]), *_rows(pu, 3),
                                          env.stream_handle(on_dev))
    L.check(st, "o3g_points_affect_panels")


def clear_inner_layer(bdry, targ, cutoff_mult=0.5 / np.sqrt(2.0 * np.pi), ips=0.01, arrays=None, stream=None):
    """clear_inner_layer method 1 (Reflect.h:446-656): push the points of `targ` (torch CUDA
    [3, n] positions) that lie below the cutoff layer of `bdry` out along the mean normal.
    Returns the number of points pushed."""
    a = arrays or bdry.device_arrays(targ.x.device)
    s = surface_struct(a)
    n = ctypes.c_int32()
    h = stream if stream is not None else ExecEnv().stream_handle(True)
    L.check(L.lib().o3g_clear_inner_layer(targ.n, *_rows(targ.x, 3), ctypes.byref(s), cutoff_mult, ips,
                                          ctypes.byref(n), h), "o3g_clear_inner_layer")
    return n.value


def represent_as_particles(bdry, offset, ts=None, bc=None, arrays=None, stream=None):
    """Surfaces::represent_as_particles (Surfaces.h:959-1008): torch CUDA (positions[3, np],
    strengths[3, np]) of one particle per panel, `offset` above the centroid along the
    normal, with the absolute panel strengths ts (default: the surface's) plus the reactive
    boundary-condition sheet (bc = (bc1, bc2)) when given."""
    a = arrays or bdry.device_arrays("cuda")
    s = surface_struct(a)
    t = a["ts"] if ts is None else ts
    npan = bdry.npanels
    px = torch.empty((3, npan), dtype=torch.float32, device=t.device)
    ps = torch.empty((3, npan), dtype=torch.float32, device=t.device)
    b1 = b2 = None
    if bc is not None:
        b1, b2 = (_base(v) for v in bc)
    h = stream if stream is not None else ExecEnv().stream_handle(True)
    L.check(L.lib().o3g_represent_as_particles(ctypes.byref(s), offset, *_rows(t, 3), b1, b2, *_rows(px, 3),
                                               *_rows(ps, 3), h), "o3g_represent_as_particles")
    return px, ps


DIFFCORES = {"gaussian": 0, "compactg": 1}


def _f32_dev(a, shape, what):
    if not (_is_dev(a) and a.dtype == torch.float32 and a.is_contiguous() and tuple(a.shape) == shape):
        raise ValueError("%s: need a contiguous float32 CUDA tensor of shape %s" % (what, shape))


def split_elongated(x, s, r, elong, core_func="gaussian", overlap=1.5, threshold=1.2, stream=None):
    """split_elongated<float> (Split.h:44-270) on torch CUDA float32 tensors x[3, n],
    s[3, n], r[n], elong[n]: every particle with elong > threshold is split in two along its
    strength, with the reference's curvature correction (core_func 'gaussian' or 'compactg',
    Core.h:27).  Returns (x, s, r, elong, nsplit): new tensors of n + nsplit particles (the
    split ones updated, their children appended in index order), or the inputs unchanged
    when nothing splits."""
    n = x.shape[1]
    for a, shp, w in ((x, (3, n), "x"), (s, (3, n), "s"), (r, (n,), "r"), (elong, (n,), "elong")):
        _f32_dev(a, shp, "split_elongated " + w)
    h = stream if stream is not None else ExecEnv().stream_handle(True)
    ns = ctypes.c_int32()
    core = DIFFCORES[core_func]
    lib = L.lib()
    st = lib.o3g_split_elongated(n, n, *_rows(x, 3), _base(r), _base(elong), *_rows(s, 3), core, overlap, threshold,
                                 ctypes.byref(ns), h)
    if st == 0:
        return x, s, r, elong, 0
    if st != 10:
        L.check(st, "o3g_split_elongated")
    cap = n + ns.value
    x2 = torch.empty((3, cap), dtype=torch.float32, device=x.device)
    s2 = torch.empty((3, cap), dtype=torch.float32, device=x.device)
    r2 = torch.empty(cap, dtype=torch.float32, device=x.device)
    e2 = torch.empty(cap, dtype=torch.float32, device=x.device)
    x2[:, :n], s2[:, :n], r2[:n], e2[:n] = x, s, r, elong
    L.check(lib.o3g_split_elongated(n, cap, *_rows(x2, 3), _base(r2), _base(e2), *_rows(s2, 3), core, overlap,
                                    threshold, ctypes.byref(ns), h), "o3g_split_elongated")
    return x2, s2, r2, e2, ns.value


def merge_close_particles(x, s, r, overlap=1.5, threshold=0.2, adapt_radii=False, stream=None):
    """merge_close_particles<float> (Merge.h:45-218) on torch CUDA float32 tensors x[3, n],
    s[3, n], r[n], merged and compacted IN PLACE (the first n - nremoved entries of each row
    hold the survivors, in order).  Returns (x, s, r, nremoved) with the survivors as new
    contiguous tensors."""
    n = x.shape[1]
    for a, shp, w in ((x, (3, n), "x"), (s, (3, n), "s"), (r, (n,), "r")):
        _f32_dev(a, shp, "merge_close_particles " + w)
    h = stream if stream is not None else ExecEnv().stream_handle(True)
    nr = ctypes.c_int32()
    L.check(L.lib().o3g_merge_close_particles(n, *_rows(x, 3), *_rows(s, 3), _base(r), overlap, threshold,
                                              int(bool(adapt_radii)), ctypes.byref(nr), h),
            "o3g_merge_close_particles")
    k = n - nr.value
    return x[:, :k].contiguous(), s[:, :k].contiguous(), r[:k].contiguous(), nr.value


def panels_on_panels_coeff(src_arrays, targ_arrays, nunk, is_self, out, ld=None, maxlev=3, stream=None):
    """Coefficients.h:169: write the column-major (ntarg*nunk) x (nsrc*nunk) block into the
    device tensor `out` (viewed with leading dimension ld, default ntarg*nunk)."""
    s = surface_struct(src_arrays)
    t = surface_struct(targ_arrays)
    ld = ld or t.np * nunk
    h = stream if stream is not None else ExecEnv().stream_handle(True)
    st = L.lib().o3g_panels_on_panels_coeff(maxlev, nunk, int(is_self), ctypes.byref(s), ctypes.byref(t),
                                            _base(out), ld, h)
    L.check(st, "o3g_panels_on_panels_coeff")


# ------------------------------------------------------------------------------------
# BEM system and solve

class BEM:
    """BEM<S,I> (BEM.h:44-234) over the device-resident system of libo3dgpu: set_block,
    set_rhs, solve, get_str.  The matrix is factorised (FP32 LU, TF32 trailing updates)
    on the first solve after it changed, and solutions are refined with FP64 residuals."""

    def __init__(self, n):
        self.n = int(n)
        h = ctypes.c_void_p()
        L.check(L.lib().o3g_bem_create(self.n, ctypes.byref(h)), "o3g_bem_create")
        self.h = h
        self.A_is_current = False
        self.factored = False
        self.b = np.zeros(self.n, np.float32)
        self.strengths = np.zeros(self.n, np.float32)
        self.iters = 0
        self.relres = float("nan")

    def __del__(self):
        try:
            if self.h:
                L.lib().o3g_bem_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def matrix(self):
        p, ld = ctypes.c_void_p(), ctypes.c_int64()
        L.check(L.lib().o3g_bem_matrix(self.h, ctypes.byref(p), ctypes.byref(ld)), "o3g_bem_matrix")
        self.factored = False
        return p.value, ld.value

    def set_block(self, rstart, cstart, blk, stream=None):
        """BEM::set_block: blk is column-major (ncols, nrows) numpy or torch CUDA."""
        ncols, nrows = blk.shape
        on = _is_dev(blk)
        L.check(L.lib().o3g_bem_set_block(self.h, rstart, nrows, cstart, ncols, _base(blk),
                                          L.MEM_DEVICE if on else L.MEM_HOST,
                                          ExecEnv(stream=stream).stream_handle(on)), "o3g_bem_set_block")
        self.factored = False

    def assemble(self, src_arrays, targ_arrays, nunk, is_self, rstart=0, cstart=0, maxlev=3, stream=None):
        """Coefficients.h:169 written straight into the system matrix at (rstart, cstart).
        A surface's block on itself on the diagonal also sets the unknowns per panel, so
        that GMRES preconditions with the panels' diagonal blocks (set_unknowns_per_panel)."""
        base, ld = self.matrix()
        s = surface_struct(src_arrays)
        t = surface_struct(targ_arrays)
        h = ExecEnv(stream=stream).stream_handle(True)
        L.check(L.lib().o3g_panels_on_panels_coeff(maxlev, nunk, int(is_self), ctypes.byref(s), ctypes.byref(t),
                                                   base + 4 * (cstart * ld + rstart), ld, h),
                "o3g_panels_on_panels_coeff")
        if is_self and rstart == cstart and rstart % nunk == 0 and self.n % nunk == 0:
            self.set_unknowns_per_panel(nunk)

    def set_unknowns_per_panel(self, bs):
        """Block size of the GMRES preconditioner (1 = none; o3g_bem_set_unknowns_per_panel)."""
        L.check(L.lib().o3g_bem_set_unknowns_per_panel(self.h, int(bs)), "o3g_bem_set_unknowns_per_panel")

    def set_rhs(self, cstart, b):
        self.b[cstart:cstart + len(b)] = _np_host(b)

    def factor(self, stream=None):
        L.check(L.lib().o3g_bem_factor(self.h, ExecEnv(stream=stream).stream_handle(True)), "o3g_bem_factor")
        self.factored = True

    def solve(self, b=None, tol=1e-10, max_iter=30, stream=None, x64=False, method="lu", restart=60):
        """BEM::solve (BEM.h:169-234); returns the FP32 strengths (and FP64 ones if asked).
        method "lu": FP32/TF32 LU (factorised once per matrix) + refinement, max_iter
        refinements; "gmres": restarted GMRES on the unfactored matrix, max_iter iterations."""
        if method not in ("lu", "gmres"):
            raise ValueError("method must be 'lu' or 'gmres'")
        if method == "lu" and not self.factored:
            self.factor(stream)
        b = self.b if b is None else b
        on = _is_dev(b)
        it, rr = ctypes.c_int32(), ctypes.c_double()
        if on:
            x = torch.empty(self.n, dtype=torch.float32, device=b.device)
            xd = torch.empty(self.n, dtype=torch.float64, device=b.device) if x64 else None
        else:
            b = np.ascontiguousarray(b, np.float32)
            x = np.empty(self.n, np.float32)
            xd = np.empty(self.n, np.float64) if x64 else None
        mem, sh = L.MEM_DEVICE if on else L.MEM_HOST, ExecEnv(stream=stream).stream_handle(on)
        if method == "lu":
            st = L.lib().o3g_bem_solve(self.h, _base(b), _base(x), None if xd is None else _base(xd), mem, tol,
                                       max_iter, ctypes.byref(it), ctypes.byref(rr), sh)
        else:
            st = L.lib().o3g_bem_solve_gmres(self.h, _base(b), _base(x), None if xd is None else _base(xd), mem,
                                             tol, max_iter, restart, ctypes.byref(it), ctypes.byref(rr), sh)
        self.iters, self.relres = it.value, rr.value
        L.check(st, "o3g_bem_solve" if method == "lu" else "o3g_bem_solve_gmres")
        if not on:
            self.strengths = x
        return (x, xd) if x64 else x

    def solve_many(self, B, tol=1e-10, max_iter=30, stream=None, x64=False, method="lu", restart=60):
        """Several right-hand sides at once: B is (nrhs, n), one right-hand side per row
        (numpy or torch CUDA float32).  Each refinement sweep / GMRES iteration streams the
        matrix once for up to 8 of them.  Returns X (nrhs, n) float32 (and the FP64 X64 if
        asked); per-column refinement or iteration counts and residuals in self.iters_many,
        self.relres_many."""
        if method not in ("lu", "gmres"):
            raise ValueError("method must be 'lu' or 'gmres'")
        if method == "lu" and not self.factored:
            self.factor(stream)
        on = _is_dev(B)
        k = int(B.shape[0])
        if B.shape != (k, self.n):
            raise ValueError("B must have shape (nrhs, %d)" % self.n)
        if on:
            B = B.contiguous().float()
            X = torch.empty((k, self.n), dtype=torch.float32, device=B.device)
            Xd = torch.empty((k, self.n), dtype=torch.float64, device=B.device) if x64 else None
        else:
            B = np.ascontiguousarray(B, np.float32)
            X = np.empty((k, self.n), np.float32)
            Xd = np.empty((k, self.n), np.float64) if x64 else None
        its = np.zeros(max(k, 1), np.int32)
        rrs = np.zeros(max(k, 1), np.float64)
        mem, sh = L.MEM_DEVICE if on else L.MEM_HOST, ExecEnv(stream=stream).stream_handle(on)
        xdp = None if Xd is None else _base(Xd)
        if method == "lu":
            st = L.lib().o3g_bem_solve_many(self.h, k, _base(B), _base(X), xdp, mem, tol, max_iter,
                                            its.ctypes.data, rrs.ctypes.data, sh)
        else:
            st = L.lib().o3g_bem_solve_gmres_many(self.h, k, _base(B), _base(X), xdp, mem, tol, max_iter, restart,
                                                  its.ctypes.data, rrs.ctypes.data, sh)
        self.iters_many, self.relres_many = its[:k].copy(), rrs[:k].copy()
        L.check(st, "o3g_bem_solve_many" if method == "lu" else "o3g_bem_solve_gmres_many")
        return (X, Xd) if x64 else X

    def get_str(self, cstart, ncols):
        return self.strengths[cstart:cstart + ncols]


def _np_host(a):
    if _is_dev(a):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def solve_bem(fs, vort, bdry, bem, env=None, maxlev=3, tol=1e-10, max_iter=30):
    """solve_bem (BEMHelper.h:43-265) for one boundary collection `bdry` (Surfaces) and a
    list of vortex-particle collections `vort` (host Points): RHS from the particles'
    panel-averaged velocity plus the freestream, the matrix assembled and factorised when
    it is not current, the FP32/TF32 LU solve refined in FP64, and the strengths scattered
    back (Surfaces::set_str, Surfaces.h:267-306)."""
    env = env or ExecEnv()
    dev = "cuda"
    arr = bdry.device_arrays(dev)
    nunk = bdry.nunk
    np_ = bdry.npanels
    pu = torch.zeros((3, np_), dtype=torch.float32, device=dev)
    for v in vort:
        src = Points(*(torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (v.x, v.s, v.r)))
        points_affect_panels(src, bdry, env, maxlev=maxlev, arrays=arr, pu=pu)
    rhs = torch.empty(np_ * nunk, dtype=torch.float32, device=dev)
    fsd = (ctypes.c_double * 3)(*fs)
    s = surface_struct(arr)
    L.check(L.lib().o3g_panel_vels_to_rhs(np_, nunk, fsd, *_rows(pu, 3), ctypes.byref(s), _base(rhs),
                                          env.stream_handle(True)), "o3g_panel_vels_to_rhs")
    if not bem.A_is_current:
        bem.assemble(arr, arr, nunk, True, maxlev=maxlev)
        bem.factor()
        bem.A_is_current = True
    x = bem.solve(rhs, tol=tol, max_iter=max_iter)
    xs = x.cpu().numpy()
    bdry.pu[...] = pu.cpu().numpy()
    bdry.set_sheet_strengths(xs[0::nunk], xs[1::nunk], xs[2::nunk] if nunk == 3 else None)
    bem.strengths = xs
    return xs


def shed_particles(fs, vort, bdry, bem, h_nu, vdelta, env=None, bc=None, maxlev=3, tol=1e-10, max_iter=30):
    """Diffusion's shedding (Diffusion.h:184-224): re-solve the BEM for the current particles
    (solve_bem), put one particle per panel 0.01 h_nu above the surface carrying the
    panel's strength (Surfaces::represent_as_particles, Surfaces.h:959-1008; bc = (bc1, bc2)
    adds the reactive boundary-condition sheet) and append them to the last collection of
    `vort` (host Points) with core radius vdelta, as Points::add_new does (Points.h:160-200);
    with no collection a new one is made.  Returns the new particles' (x, s) [3, np]."""
    solve_bem(fs, vort, bdry, bem, env, maxlev, tol, max_iter)
    # the reference's offset 0.01*(S)h_nu: double product rounded to the float parameter
    offset = float(np.float32(0.01 * float(np.float32(h_nu))))
    px, ps = represent_as_particles(bdry, offset, bc=bc, arrays=bdry.device_arrays("cuda"))
    x, s = px.cpu().numpy(), ps.cpu().numpy()
    r = np.full(x.shape[1], np.float32(vdelta), np.float32)
    if vort:
        v = vort[-1]
        v.x = np.ascontiguousarray(np.concatenate([v.x, x], axis=1))
        v.s = np.ascontiguousarray(np.concatenate([v.s, s], axis=1))
        v.r = np.ascontiguousarray(np.concatenate([v.r, r]))
        grads = v.ug is not None
        v.u = np.zeros((3, v.x.shape[1]), np.float32)
        v.ug = np.zeros((9, v.x.shape[1]), np.float32) if grads else None
    else:
        vort.append(Points(x, s, r))
    return x, s


# ------------------------------------------------------------------------------------
# convection

def _ptrs(t, k):
    return (ctypes.c_void_p * k)(*_rows(t, k))


class Ralston:
    """Convection::advect_2nd_ralston (Convection.h:349-425) for a boundary-free set of
    vortex particles held in torch CUDA tensors x[3,n], s[3,n], r[n], elong[n] (advanced in
    place) and optional field points f[3,nf].  Each step: two vel+grad evaluations, the
    2/3 dt interim Euler move with stretching, and the 0.25/0.75 combine.  Steps after the
    first replay a captured CUDA graph."""

    def __init__(self, x, s, r, elong, fieldpts=None, env=None, use_graph=True):
        env = env or ExecEnv()
        self.x, self.s, self.r, self.elong, self.f = x, s, r, elong, fieldpts
        self.stream = torch.cuda.Stream(device=x.device) if use_graph else torch.cuda.current_stream(x.device)
        h = ctypes.c_void_p()
        nf = 0 if fieldpts is None else fieldpts.shape[1]
        L.check(L.lib().o3g_rk2_create(L.CORES[env.core], L.PRECS[env.precision], x.shape[1], _ptrs(x, 3),
                                       _ptrs(s, 3), _base(r), _base(elong), nf,
                                       _ptrs(fieldpts, 3) if nf else None, int(use_graph), ctypes.byref(h)),
                "o3g_rk2_create")
        self.h = h

    def step(self, dt, fs=(0.0, 0.0, 0.0), nsteps=1):
        fsd = (ctypes.c_double * 3)(*fs)
        self.stream.wait_stream(torch.cuda.current_stream(self.x.device))
        L.check(L.lib().o3g_rk2_step(self.h, dt, fsd, nsteps, self.stream.cuda_stream), "o3g_rk2_step")
        torch.cuda.current_stream(self.x.device).wait_stream(self.stream)

    def attach_body(self, surfaces, bem, maxlev=3, tol=1e-10, max_iter=30, ips=0.0, arrays=None):
        """Adds a fixed body (Surfaces) whose BEM system (`bem`, np * nunk unknowns) is solved
        at every stage for that stage's particles (solve_bem inside find_derivs,
        Convection.h:188-202); with ips > 0 points are pushed out of the body after each move
        (clear_inner_layer, Convection.h:372,381,423-424).  Steps then run directly."""
        self.body_arrays = arrays or surfaces.device_arrays(self.x.device)
        self.body_struct = surface_struct(self.body_arrays)
        self.body_bem = bem
        L.check(L.lib().o3g_rk2_attach_body(self.h, ctypes.byref(self.body_struct), surfaces.nunk, maxlev, bem.h,
                                            tol, max_iter, ips, self.stream.cuda_stream), "o3g_rk2_attach_body")

    def body_stats(self):
        n, it, rr, mx, pu = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        L.check(L.lib().o3g_rk2_body_stats(self.h, ctypes.byref(n), ctypes.byref(it), ctypes.byref(rr),
                                           ctypes.byref(mx), ctypes.byref(pu)), "o3g_rk2_body_stats")
        return {"solves": n.value, "last_refinements": it.value, "last_relres": rr.value, "max_relres": mx.value,
                "pushed": pu.value}

    def body_strengths(self):
        """(ts[3, np], solution[np * nunk]) of the last stage solved, as numpy arrays."""
        npan = self.body_struct.np
        ts = np.zeros((3, npan), np.float32)
        sol = np.zeros(self.body_bem.n, np.float32)
        L.check(L.lib().o3g_rk2_body_strengths(self.h, (ctypes.c_void_p * 3)(*_rows(ts, 3)), sol.ctypes.data,
                                               self.stream.cuda_stream), "o3g_rk2_body_strengths")
        return ts, sol

    def velocities(self):
        """Stage-1 velocity and gradient device pointers of the last step (u[3], ug[9])."""
        u = (ctypes.c_void_p * 3)()
        g = (ctypes.c_void_p * 9)()
        L.check(L.lib().o3g_rk2_velocities(self.h, u, g), "o3g_rk2_velocities")
        return list(u), list(g)

    def __del__(self):
        try:
            if self.h:
                L.lib().o3g_rk2_destroy(self.h)
                self.h = None
        except Exception:
            pass


# ------------------------------------------------------------------------------------
# many independent systems in one launch

class BatchSystem:
    """One independent particle system of a batch, on the device: particles x[3,np],
    s[3,np], r[np] with result arrays u[3,np] (+ ug[9,np]), and optional field points
    f[3,nf] with fu[3,nf] (+ fug[9,nf]).  Results accumulate (+=)."""

    def __init__(self, x, s, r, u, ug=None, f=None, fu=None, fug=None):
        self.x, self.s, self.r, self.u, self.ug = x, s, r, u, ug
        self.f, self.fu, self.fug = f, fu, fug

    def struct(self, grads):
        st = L.System()
        n = self.x.shape[1]
        for t, k in ((self.x, 3), (self.s, 3), (self.u, 3)):
            if not (_is_dev(t) and t.dtype == torch.float32 and t.is_contiguous() and tuple(t.shape) == (k, n)):
                raise ValueError("batch system arrays must be contiguous float32 CUDA tensors [k, np]")
        st.np = n
        st.x, st.y, st.z = _rows(self.x, 3)
        st.r = _base(self.r)
        st.sx, st.sy, st.sz = _rows(self.s, 3)
        st.u, st.v, st.w = _rows(self.u, 3)
        if grads:
            for k, p in enumerate(_rows(self.ug, 9)):
                st.ug[k] = p
        nf = 0 if self.f is None else self.f.shape[1]
        st.nf = nf
        if nf:
            st.fx, st.fy, st.fz = _rows(self.f, 3)
            st.fu, st.fv, st.fw = _rows(self.fu, 3)
            if grads:
                for k, p in enumerate(_rows(self.fug, 9)):
                    st.fug[k] = p
        return st


class Batch:
    """Pair sums of many independent systems (BatchSystem) in one persistent launch per
    run, with autotuned, per-shape cached configuration (o3g_batch_*)."""

    def __init__(self, systems, env=None, grads=True):
        env = env or ExecEnv()
        self.env, self.grads, self.systems = env, grads, list(systems)
        arr = (L.System * len(self.systems))(*[s.struct(grads) for s in self.systems])
        h = ctypes.c_void_p()
        L.check(L.lib().o3g_batch_create(L.CORES[env.core], L.PRECS[env.precision], int(grads), len(self.systems),
                                         arr, ctypes.byref(h)), "o3g_batch_create")
        self.h = h

    def run(self, stream=None):
        st = stream if stream is not None else self.env.stream_handle(True)
        if torch is not None and isinstance(st, torch.cuda.Stream):
            st = st.cuda_stream
        L.check(L.lib().o3g_batch_run(self.h, st), "o3g_batch_run")

    def tune(self, stream=None):
        st = stream if stream is not None else self.env.stream_handle(True)
        L.check(L.lib().o3g_batch_tune(self.h, st), "o3g_batch_tune")

    def set_config(self, tpt, blocks_per_sm=0, split=4):
        L.check(L.lib().o3g_batch_set_config(self.h, tpt, blocks_per_sm, split), "o3g_batch_set_config")

    def config(self):
        v = [ctypes.c_int32() for _ in range(6)]
        L.check(L.lib().o3g_batch_get_config(self.h, *[ctypes.byref(x) for x in v]), "o3g_batch_get_config")
        return dict(zip(("tpt", "grid", "split", "chunk", "nitems", "tuned"), [x.value for x in v]))

    def __del__(self):
        try:
            if self.h:
                L.lib().o3g_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass


class BatchRalston(Ralston):
    """Ralston RK2 of many independent systems stored back to back in x[3,N], s[3,N], r[N],
    elong[N] (system i owns np[i] consecutive particles) and field points f[3,NF] (nf[i]
    each); both evaluations of a step are one batched persistent launch each."""

    def __init__(self, np_counts, nf_counts, x, s, r, elong, fieldpts=None, env=None, use_graph=True):
        env = env or ExecEnv()
        self.x, self.s, self.r, self.elong, self.f = x, s, r, elong, fieldpts
        self.stream = torch.cuda.Stream(device=x.device) if use_graph else torch.cuda.current_stream(x.device)
        nsys = len(np_counts)
        npa = (ctypes.c_int32 * nsys)(*[int(v) for v in np_counts])
        nfa = (ctypes.c_int32 * nsys)(*[int(v) for v in nf_counts])
        if sum(np_counts) != x.shape[1] or (sum(nf_counts) != (0 if fieldpts is None else fieldpts.shape[1])):
            raise ValueError("per-system counts do not add up to the array sizes")
        h = ctypes.c_void_p()
        L.check(L.lib().o3g_batch_rk2_create(L.CORES[env.core], L.PRECS[env.precision], nsys, npa, nfa, _ptrs(x, 3),
                                             _ptrs(s, 3), _base(r), _base(elong),
                                             _ptrs(fieldpts, 3) if sum(nf_counts) else None, int(use_graph),
                                             ctypes.byref(h)), "o3g_batch_rk2_create")
        self.h = h
