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
    for m in re.finditer(r"\b(o3g_[a-z0-9_]+)\s*\(([^;{}]*?)\)\s*;", txt, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


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
