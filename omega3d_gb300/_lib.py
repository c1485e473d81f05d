"""ctypes binding of libo3dgpu.so (the C-ABI declared in include/o3dgpu.h).

The library is built in-tree by omega3d_gb300/build.py.  Loading fails loudly when
it is missing: there is no CPU fallback behind this package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libo3dgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "o3dgpu.h")

O3G_OK = 0
STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "no usable sm_103 device",
    4: "device allocation failed", 5: "iterative refinement did not converge", 6: "device-side wait timed out",
    7: "singular or non-finite pivot", 8: "non-finite input", 9: "call made in the wrong state",
    10: "output arrays too small",
}
CORES = {"rm": 0, "wl": 1, "exp": 2, "gauss": 3, "v2": 4}
PRECS = {"plain": 0, "compensated": 1, "fp64": 2, "accurate": 3}
MEM_HOST, MEM_DEVICE = 0, 1

_lib = None

c_i32 = ctypes.c_int32
c_vp = ctypes.c_void_p
c_f = ctypes.c_float
c_d = ctypes.c_double


class O3GError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = "%s failed: %s" % (where, STATUS.get(status, "status %d" % status))
        try:
            detail = lib().o3g_last_error().decode()
            if detail:
                msg += " (%s)" % detail
        except Exception:  # pragma: no cover - loading problems are reported elsewhere
            pass
        super().__init__(msg)


class Surface(ctypes.Structure):
    """o3g_surface_t (include/o3dgpu.h)."""
    _fields_ = [("nn", ctypes.c_int32), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("np", ctypes.c_int32), ("idx", ctypes.c_void_p), ("area", ctypes.c_void_p),
                ("x1x", ctypes.c_void_p), ("x1y", ctypes.c_void_p), ("x1z", ctypes.c_void_p),
                ("x2x", ctypes.c_void_p), ("x2y", ctypes.c_void_p), ("x2z", ctypes.c_void_p),
                ("nx", ctypes.c_void_p), ("ny", ctypes.c_void_p), ("nz", ctypes.c_void_p)]


class System(ctypes.Structure):
    """o3g_system_t (include/o3dgpu.h): one independent particle system of a batch."""
    _fields_ = [("np", ctypes.c_int32), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("r", ctypes.c_void_p), ("sx", ctypes.c_void_p), ("sy", ctypes.c_void_p), ("sz", ctypes.c_void_p),
                ("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("w", ctypes.c_void_p), ("ug", ctypes.c_void_p * 9),
                ("nf", ctypes.c_int32), ("fx", ctypes.c_void_p), ("fy", ctypes.c_void_p), ("fz", ctypes.c_void_p),
                ("fu", ctypes.c_void_p), ("fv", ctypes.c_void_p), ("fw", ctypes.c_void_p), ("fug", ctypes.c_void_p * 9)]


def _declare(l):
    P = c_vp
    l.o3g_status_string.restype = ctypes.c_char_p
    l.o3g_status_string.argtypes = [c_i32]
    l.o3g_last_error.restype = ctypes.c_char_p
    l.o3g_last_error.argtypes = []
    l.o3g_version.restype = c_i32
    l.o3g_version.argtypes = []
    l.o3g_device_info.restype = c_i32
    l.o3g_device_info.argtypes = [P, P, P, P]
    l.o3g_flops_per_pair.restype = c_i32
    l.o3g_flops_per_pair.argtypes = [c_i32, c_i32, c_i32]
    l.o3g_set_timing.restype = c_i32
    l.o3g_set_timing.argtypes = [c_i32]
    l.o3g_last_kernel_ms.restype = c_i32
    l.o3g_last_kernel_ms.argtypes = [P]
    l.o3g_launch_count.restype = c_i32
    l.o3g_launch_count.argtypes = [P]
    l.o3g_alloc_count.restype = c_i32
    l.o3g_alloc_count.argtypes = [P]
    l.o3g_debug_wait_test.restype = c_i32
    l.o3g_debug_wait_test.argtypes = [c_i32]
    l.o3g_fp32_peak_probe.restype = c_i32
    l.o3g_fp32_peak_probe.argtypes = [c_i32, P, P, P]
    l.o3g_exp_probe.restype = c_i32
    l.o3g_exp_probe.argtypes = [c_i32, P, P, P]
    l.o3g_div3_check.restype = c_i32
    l.o3g_div3_check.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), P]
    l.o3g_gemm_tf32_sub.restype = c_i32
    l.o3g_gemm_tf32_sub.argtypes = [c_i32, c_i32, c_i32, P, ctypes.c_int64, P, ctypes.c_int64, P, ctypes.c_int64, P]
    l.o3g_points_affect_points.restype = c_i32
    l.o3g_points_affect_points.argtypes = [c_i32, c_i32, c_i32, c_i32] + [P] * 7 + [c_i32] + [P] * 4 + [P] * 3 + [P, P]
    for name in ("external_vel_solver_f_", "external_vel_solver_d_"):
        fn = getattr(l, name)
        fn.argtypes = [P] * 24
        fn.restype = c_f
    l.o3g_external_set_method.argtypes = [c_i32, c_i32]
    l.o3g_external_set_method.restype = c_i32
    l.o3g_external_get_method.argtypes = [P, P]
    l.o3g_external_get_method.restype = c_i32
    l.o3g_ovoid_size.restype = c_i32
    l.o3g_ovoid_size.argtypes = [c_i32, P, P]
    l.o3g_generate_ovoid.restype = c_i32
    l.o3g_generate_ovoid.argtypes = [c_i32, c_f, c_f, c_f, P, P, P, P]
    l.o3g_compute_bases.restype = c_i32
    l.o3g_compute_bases.argtypes = [c_i32, P, P, P, c_i32, P] + [P] * 10
    l.o3g_sheet_to_panel_strength.restype = c_i32
    l.o3g_sheet_to_panel_strength.argtypes = [c_i32] + [P] * 12
    l.o3g_panels_affect_points.restype = c_i32
    l.o3g_panels_affect_points.argtypes = [c_i32, c_i32, c_i32, c_i32, P, P, P, c_i32, P, P, P, P, P, P, c_i32, P, P, P,
                                           P, P, P, P, P]
    l.o3g_points_affect_panels.restype = c_i32
    l.o3g_points_affect_panels.argtypes = [c_i32, c_i32, c_i32, c_i32] + [P] * 6 + [c_i32, P, P, P, c_i32, P, P, P, P, P,
                                                                           P]
    l.o3g_panels_on_panels_coeff.restype = c_i32
    l.o3g_panels_on_panels_coeff.argtypes = [c_i32, c_i32, c_i32, P, P, P, ctypes.c_int64, P]
    l.o3g_bem_create.restype = c_i32
    l.o3g_bem_create.argtypes = [ctypes.c_int64, P]
    l.o3g_bem_destroy.restype = c_i32
    l.o3g_bem_destroy.argtypes = [P]
    l.o3g_bem_matrix.restype = c_i32
    l.o3g_bem_matrix.argtypes = [P, P, P]
    l.o3g_bem_set_block.restype = c_i32
    l.o3g_bem_set_block.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, P, c_i32, P]
    l.o3g_bem_factor.restype = c_i32
    l.o3g_bem_factor.argtypes = [P, P]
    l.o3g_bem_solve.restype = c_i32
    l.o3g_bem_solve.argtypes = [P, P, P, P, c_i32, c_d, c_i32, P, P, P]
    l.o3g_bem_solve_gmres.restype = c_i32
    l.o3g_bem_solve_gmres.argtypes = [P, P, P, P, c_i32, c_d, c_i32, c_i32, P, P, P]
    l.o3g_bem_set_unknowns_per_panel.restype = c_i32
    l.o3g_bem_set_unknowns_per_panel.argtypes = [P, c_i32]
    l.o3g_bem_solve_many.restype = c_i32
    l.o3g_bem_solve_many.argtypes = [P, c_i32, P, P, P, c_i32, c_d, c_i32, P, P, P]
    l.o3g_bem_solve_gmres_many.restype = c_i32
    l.o3g_bem_solve_gmres_many.argtypes = [P, c_i32, P, P, P, c_i32, c_d, c_i32, c_i32, P, P, P]
    l.o3g_panel_vels_to_rhs.restype = c_i32
    l.o3g_panel_vels_to_rhs.argtypes = [c_i32, c_i32, P, P, P, P, P, P, P]
    l.o3g_points_finalize.restype = c_i32
    l.o3g_points_finalize.argtypes = [c_i32, P, P, P, P]
    l.o3g_points_move_euler.restype = c_i32
    l.o3g_points_move_euler.argtypes = [c_i32, c_d, c_d, P, P, P, P, P, P]
    l.o3g_points_move_rk2.restype = c_i32
    l.o3g_points_move_rk2.argtypes = [c_i32, c_d, c_d, P, P, c_d, P, P, P, P, P, P]
    l.o3g_rk2_create.restype = c_i32
    l.o3g_rk2_create.argtypes = [c_i32, c_i32, c_i32, P, P, P, P, c_i32, P, c_i32, P]
    l.o3g_rk2_step.restype = c_i32
    l.o3g_rk2_step.argtypes = [P, c_d, P, c_i32, P]
    l.o3g_rk2_velocities.restype = c_i32
    l.o3g_rk2_velocities.argtypes = [P, P, P]
    l.o3g_rk2_destroy.restype = c_i32
    l.o3g_rk2_destroy.argtypes = [P]
    l.o3g_rk2_attach_body.restype = c_i32
    l.o3g_rk2_attach_body.argtypes = [P, P, c_i32, c_i32, P, c_d, c_i32, c_f, P]
    l.o3g_rk2_body_stats.restype = c_i32
    l.o3g_rk2_body_stats.argtypes = [P, P, P, P, P, P]
    l.o3g_represent_as_particles.restype = c_i32
    l.o3g_represent_as_particles.argtypes = [P, c_f] + [P] * 11 + [P]
    l.o3g_clear_inner_layer.restype = c_i32
    l.o3g_clear_inner_layer.argtypes = [c_i32, P, P, P, P, c_f, c_f, P, P]
    l.o3g_panels_affect_panels.restype = c_i32
    l.o3g_panels_affect_panels.argtypes = [c_i32, c_i32, c_i32, c_i32, P, P, P, c_i32, P, P, P, P, P, P,
                                           c_i32, P, P, P, c_i32, P, P, P, P, P, P, P, P]
    l.o3g_split_elongated.restype = c_i32
    l.o3g_split_elongated.argtypes = [c_i32, c_i32] + [P] * 8 + [c_i32, c_f, c_f, P, P]
    l.o3g_merge_close_particles.restype = c_i32
    l.o3g_merge_close_particles.argtypes = [c_i32] + [P] * 7 + [c_f, c_f, c_i32, P, P]
    l.o3g_rk2_body_strengths.restype = c_i32
    l.o3g_rk2_body_strengths.argtypes = [P, P, P, P]
    l.o3g_bem_size.restype = c_i32
    l.o3g_bem_size.argtypes = [P, P]
    l.o3g_points_affect_points_noalloc.restype = c_i32
    l.o3g_points_affect_points_noalloc.argtypes = [c_i32, c_i32, c_i32] + [P] * 7 + [c_i32] + [P] * 4 + [P] * 3 + [P, P]
    l.o3g_batch_create.restype = c_i32
    l.o3g_batch_create.argtypes = [c_i32, c_i32, c_i32, c_i32, P, P]
    l.o3g_batch_run.restype = c_i32
    l.o3g_batch_run.argtypes = [P, P]
    l.o3g_batch_tune.restype = c_i32
    l.o3g_batch_tune.argtypes = [P, P]
    l.o3g_batch_set_config.restype = c_i32
    l.o3g_batch_set_config.argtypes = [P, c_i32, c_i32, c_i32]
    l.o3g_batch_get_config.restype = c_i32
    l.o3g_batch_get_config.argtypes = [P, P, P, P, P, P, P]
    l.o3g_batch_destroy.restype = c_i32
    l.o3g_batch_destroy.argtypes = [P]
    l.o3g_batch_velgrad.restype = c_i32
    l.o3g_batch_velgrad.argtypes = [c_i32, c_i32, c_i32, c_i32, P, P]
    l.o3g_batch_plan.restype = c_i32
    l.o3g_batch_plan.argtypes = [c_i32, P, P, c_i32, c_i32, c_i32, P, P, P, P, P, P]
    l.o3g_batch_rk2_create.restype = c_i32
    l.o3g_batch_rk2_create.argtypes = [c_i32, c_i32, c_i32, P, P, P, P, P, P, P, c_i32, P]
    l.o3g_points_affect_points_d.restype = c_i32
    l.o3g_points_affect_points_d.argtypes = [c_i32, c_i32, c_i32] + [P] * 7 + [c_i32] + [P] * 4 + [P] * 3 + [P, P]


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libo3dgpu.so not built at %s; run omega3d_gb300/build.py "
                              "(or __graft_entry__.build())" % LIB_PATH)
        l = ctypes.CDLL(LIB_PATH)
        _declare(l)
        _lib = l
    return _lib


def check(status, where):
    if status != O3G_OK:
        raise O3GError(status, where)


def launch_count():
    n = ctypes.c_uint64(0)
    check(lib().o3g_launch_count(ctypes.byref(n)), "o3g_launch_count")
    return int(n.value)


def header_symbols():
    """Names of every entry point declared in include/o3dgpu.h."""
    import re
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(o3g_[a-z0-9_]+|external_vel_solver_[fd]_)\s*\(", txt)))
