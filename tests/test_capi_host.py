"""CPU-only checks of the C-ABI library: it loads, exports every symbol that
include/mglc.h declares, and rejects bad parameters before touching the GPU."""
import ctypes
import os
import re

import pytest

from mglc_gb300 import build as B
from mglc_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "mglc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mglc_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return capi.lib()


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    # the Python binding declares the same set
    assert set(names) == set(capi.SIGNATURES)


def test_invalid_parameters_are_rejected_without_a_gpu(lib):
    ctx = ctypes.c_void_p()
    p = capi.LidParams(1, 8, 8, 400.0, 1.0, 0.1, 1, 0)
    rc = lib.mglc_lid_create(ctypes.byref(p), ctypes.byref(ctx))
    assert rc == 1
    assert b"at least 2" in lib.mglc_last_error(ctx)
    lib.mglc_destroy(ctx)
    p = capi.LidParams(8, 8, 8, -1.0, 1.0, 0.1, 1, 0)
    ctx = ctypes.c_void_p()
    assert lib.mglc_lid_create(ctypes.byref(p), ctypes.byref(ctx)) == 1
    lib.mglc_destroy(ctx)
    p = capi.LidParams(8, 8, 8, 400.0, 1.0, 0.1, 1, 9)
    ctx = ctypes.c_void_p()
    assert lib.mglc_lid_create(ctypes.byref(p), ctypes.byref(ctx)) == 1
    assert b"precision" in lib.mglc_last_error(ctx)
    lib.mglc_destroy(ctx)
    t = capi.ThermalParams(8, 8, 8, -1.0, 0.71, 0.1, 0.5, -0.5, 0.0, 0.0, 1, 0, 0)
    ctx = ctypes.c_void_p()
    assert lib.mglc_thermal_create(ctypes.byref(t), ctypes.byref(ctx)) == 1
    lib.mglc_destroy(ctx)


def test_null_arguments(lib):
    assert lib.mglc_lid_create(None, None) == 1
    assert lib.mglc_step(None, 1) == 1
    assert lib.mglc_last_error(None) == b"null context"
    lib.mglc_destroy(None)


def test_lid2d_parameters_are_rejected_without_a_gpu(lib):
    for args, rc_want, msg in (((1, 8, 400.0, 1.0, 0.1, 0), 1, b"nx, ny"),
                               ((8, 8, -5.0, 1.0, 0.1, 0), 1, b"reynolds"),
                               ((8, 8, 400.0, 1.0, 0.1, 1), 6, b"MGLC_FP64")):
        ctx = ctypes.c_void_p()
        p = capi.Lid2DParams(*args)
        assert lib.mglc_lid2d_create(ctypes.byref(p), ctypes.byref(ctx)) == rc_want
        assert msg in lib.mglc_last_error(ctx)
        lib.mglc_destroy(ctx)


def test_shear2d_parameters_are_rejected_without_a_gpu(lib):
    import numpy as np
    for args, centers, msg in (((4, 40, 0.8, 1.0, 2.0, 5.0, 0.02, 0.1, 0, 0), [[20.0, 20.0]], b"nx, ny"),
                               ((64, 40, 0.5, 1.0, 2.0, 5.0, 0.02, 0.1, 0, 0), [[20.0, 20.0]], b"tauf"),
                               ((64, 40, 0.8, 1.0, 2.0, 5.0, 0.02, 0.1, 0, 0), [[4.0, 20.0]],
                                b"periodic boundary")):
        ctx = ctypes.c_void_p()
        c = np.ascontiguousarray(centers, dtype=np.float64)
        p = capi.Shear2DParams(*args)
        assert lib.mglc_shear2d_create(ctypes.byref(p), c.ctypes.data, len(c), ctypes.byref(ctx)) == 1
        assert msg in lib.mglc_last_error(ctx)
        lib.mglc_destroy(ctx)


def test_sequential_sum_rejects_bad_arguments_without_a_gpu(lib):
    import numpy as np
    x = np.ones(4)
    keep = np.ones(4, np.int32)
    s, n = ctypes.c_double(), ctypes.c_longlong()
    f = lib.mglc_sequential_sum
    assert f(x.ctypes.data, keep.ctypes.data, -1, ctypes.byref(s), ctypes.byref(n)) == 1
    assert f(None, keep.ctypes.data, 4, ctypes.byref(s), ctypes.byref(n)) == 1
    assert f(x.ctypes.data, None, 4, ctypes.byref(s), ctypes.byref(n)) == 1
    assert f(x.ctypes.data, keep.ctypes.data, 4, None, ctypes.byref(n)) == 1
    assert f(x.ctypes.data, keep.ctypes.data, 4, ctypes.byref(s), None) == 1
