"""CPU tests of the C-ABI library: it loads, exports every entry point declared in
include/o3dgpu.h, and validates arguments before touching a device."""
import ctypes

import numpy as np
import pytest

from omega3d_gb300 import _lib as L


def test_every_declared_symbol_is_exported(built_lib):
    names = L.header_symbols()
    assert "o3g_points_affect_points" in names
    missing = [n for n in names if not hasattr(built_lib, n)]
    assert not missing, "declared but not exported: %s" % missing


def test_status_strings(built_lib):
    for code, text in L.STATUS.items():
        assert built_lib.o3g_status_string(code).decode() == text
    assert built_lib.o3g_version() >= 100


def test_flop_counts(built_lib):
    assert built_lib.o3g_flops_per_pair(0, 1, 1) == 63
    assert built_lib.o3g_flops_per_pair(0, 1, 0) == 61
    assert built_lib.o3g_flops_per_pair(1, 1, 1) == 70
    assert built_lib.o3g_flops_per_pair(2, 1, 1) == 68
    assert built_lib.o3g_flops_per_pair(9, 1, 1) == -1


def _call(lib, core=0, prec=0, mem=0, ns=4, nt=4, null_src=False, grads=True):
    a = np.zeros((3, max(ns, 1)), np.float32)
    r = np.ones(max(ns, 1), np.float32)
    u = np.zeros((3, max(nt, 1)), np.float32)
    g = np.zeros((9, max(nt, 1)), np.float32)
    P = lambda arr, k=0: arr.ctypes.data + k * arr.shape[-1] * 4  # noqa: E731
    src = [None] * 7 if null_src else [P(a, 0), P(a, 1), P(a, 2), P(r), P(a, 0), P(a, 1), P(a, 2)]
    tug = (ctypes.c_void_p * 9)(*[P(g, k) for k in range(9)]) if grads else None
    return lib.o3g_points_affect_points(core, prec, mem, ns, *src, nt, P(a, 0), P(a, 1), P(a, 2), P(r),
                                        P(u, 0), P(u, 1), P(u, 2), tug, None)


def test_argument_validation_without_device(built_lib):
    assert _call(built_lib, core=7) == 1
    assert _call(built_lib, prec=5) == 1
    assert _call(built_lib, mem=3) == 1
    assert _call(built_lib, ns=-1) == 1
    assert _call(built_lib, null_src=True) == 1
    # empty problems are a successful no-op and need no device
    assert _call(built_lib, ns=0) == 0
    assert _call(built_lib, nt=0) == 0


def test_no_device_is_reported_not_crashed(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    st = _call(built_lib)
    assert st in (2, 3)


def _prototypes():
    """{name: number of parameters} of every function declared in include/o3dgpu.h."""
    import re
    txt = open(L.HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for m in re.finditer(r"\b(o3g_[a-z0-9_]+|external_vel_solver_[fd]_)\s*\(([^;{}]*?)\)\s*;", txt, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_every_entry_point_has_declared_argument_types(built_lib):
    """A ctypes call without argtypes passes Python ints as 32-bit C ints, which truncates
    device pointers: every entry point of the header must have its argument types declared."""
    missing = [n for n in L.header_symbols() if getattr(built_lib, n).argtypes is None]
    assert not missing, missing


def test_bindings_match_header_prototypes(built_lib):
    """Every entry point the Python binding declares argtypes for takes as many arguments
    as its C prototype (a miscounted argtypes list would shift every later pointer)."""
    protos = _prototypes()
    assert len(protos) >= 40
    checked, bad = 0, []
    for name, nargs in protos.items():
        fn = getattr(built_lib, name)
        if fn.argtypes is None:
            continue
        checked += 1
        if len(fn.argtypes) != nargs:
            bad.append((name, nargs, len(fn.argtypes)))
    assert not bad, "argtypes count differs from the prototype: %s" % bad
    assert checked >= 30


def test_external_hook_method_and_validation(built_lib):
    """The reference's hook symbols: method selection, and the checks made before any
    device is touched (null counts; an empty source set adds nothing and still returns the
    reference's per-target flop count)."""
    c, p = ctypes.c_int32(), ctypes.c_int32()
    assert built_lib.o3g_external_set_method(-1, -1) == 0
    assert built_lib.o3g_external_get_method(ctypes.byref(c), ctypes.byref(p)) == 0
    import os
    if "O3G_EXTERNAL_CORE" not in os.environ and "O3G_EXTERNAL_PREC" not in os.environ:
        assert (c.value, p.value) == (1, 0)          # WL, PLAIN: CoreFunc.h:37 and the float path
    assert built_lib.o3g_external_set_method(0, 1) == 0
    assert built_lib.o3g_external_get_method(ctypes.byref(c), ctypes.byref(p)) == 0
    assert (c.value, p.value) == (0, 1)
    assert built_lib.o3g_external_set_method(7, 0) == 1
    assert built_lib.o3g_external_set_method(-1, -1) == 0
    nul = [None] * 22
    assert built_lib.external_vel_solver_f_(None, *nul, None) == -1.0
    ns, nt = ctypes.c_int(0), ctypes.c_int(5)
    t = np.zeros(5, np.float32)
    args = [ctypes.byref(ns)] + [None] * 7 + [ctypes.byref(nt)] + [t.ctypes.data] * 15
    assert built_lib.external_vel_solver_f_(*args) == 5 * 12.0
    td = np.zeros(5, np.float64)
    args = [ctypes.byref(ns)] + [None] * 7 + [ctypes.byref(nt)] + [td.ctypes.data] * 15
    assert built_lib.external_vel_solver_d_(*args) == 5 * 12.0


def test_reference_hook_declarations_compile_against_the_header(built_lib, tmp_path):
    """The reference's own EXTERNAL_VEL_SOLVE declarations (Influence.h:33-48), compiled in
    one C++ translation unit with include/o3dgpu.h and linked with libo3dgpu.so: a
    declaration whose types differed from the library's would not compile (two extern "C"
    declarations of one name must agree).  Needs the reference sources beside this checkout."""
    import os
    import re
    import subprocess
    src = os.environ.get("O3D_REFERENCE_SRC") or os.path.join(
        os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(L.HEADER)))), "reference", "src")
    path = os.path.join(src, "Influence.h")
    if not os.path.exists(path):
        pytest.skip("reference sources not present")
    txt = open(path).read()
    m = re.search(r"#ifdef EXTERNAL_VEL_SOLVE\n(.*?)#endif", txt, flags=re.S)
    assert m and "external_vel_solver_f_" in m.group(1)
    tu = tmp_path / "hook.cpp"
    tu.write_text('#include "o3dgpu.h"\n' + m.group(1) + '''
int main() {
  int ns = 0, nt = 0;
  float* p = nullptr;
  return (int)external_vel_solver_f_(&ns, p, p, p, p, p, p, p, &nt, p, p, p,
                                     p, p, p, p, p, p, p, p, p, p, p, p);
}
''')
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.dirname(L.HEADER), str(tu), "-o", str(tmp_path / "hook"),
                        L.LIB_PATH, "-Wl,--unresolved-symbols=ignore-in-shared-libs"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
