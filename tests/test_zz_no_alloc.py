"""The no-allocation residual entry point (mglc_residual_noalloc).

It serves callers that cannot allocate device memory (hosts whose device
memory belongs to another runtime's fixed pool, or loops that must not pay
cudaMalloc's implicit synchronisation): they pass their own device arrays and
the reduction uses a static device array instead of a cudaMalloc'd one.
These tests check it against the context-based mglc_check on two calls in a
row.  This file sorts last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from mglc_gb300 import build as B
from mglc_gb300 import capi


def _noalloc(L, n, u, v, w, T, up, vp, wp, Tp, with_w, stream):
    eu, et = ctypes.c_double(), ctypes.c_double()
    buf = ctypes.create_string_buffer(256)
    p = lambda t: None if t is None else t.data_ptr()
    rc = L.mglc_residual_noalloc(n, p(u), p(v), p(w), p(T), p(up), p(vp), p(wp), p(Tp), with_w,
                                 stream, ctypes.byref(eu), ctypes.byref(et), buf, 256)
    assert rc == 0, buf.value.decode()
    return eu.value, et.value


def test_rejects_sizes_beyond_the_static_limit():
    B.build()
    L = capi.lib()
    buf = ctypes.create_string_buffer(256)
    eu = ctypes.c_double()
    dummy = ctypes.c_void_p(16)
    rc = L.mglc_residual_noalloc(67108864 + 1, dummy, dummy, dummy, None, dummy, dummy, dummy,
                                 None, 0, None, ctypes.byref(eu), None, buf, 256)
    assert rc == 1 and b"exceeds the static scratch limit" in buf.value


@pytest.mark.gpu
def test_noalloc_residual_matches_check_lid_two_calls():
    import torch
    import mglc_gb300
    B.build()
    L = capi.lib()
    nx, ny, nz = 24, 20, 16
    n = nx * ny * nz
    dev = lambda: torch.empty(n, dtype=torch.float64, device="cuda")
    u, v, w = dev(), dev(), dev()
    up, vp, wp = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
    stream = torch.cuda.Stream()
    with mglc_gb300.LidDrivenCavity(nx, ny, nz, reynolds=100.0, u0=0.1) as c:
        c.initial()
        for call in range(2):
            c.step(25)
            rc = L.mglc_get_macros_device(c.handle, None, u.data_ptr(), v.data_ptr(),
                                          w.data_ptr(), None)
            assert rc == 0
            ref = c.check()
            got, _ = _noalloc(L, n, u, v, w, None, up, vp, wp, None, 0, stream.cuda_stream)
            np.testing.assert_allclose(got, ref, rtol=1e-9)
            assert torch.equal(up, u) and torch.equal(wp, w)


@pytest.mark.gpu
def test_noalloc_residual_matches_check_thermal_two_calls():
    import torch
    import mglc_gb300
    B.build()
    L = capi.lib()
    nx, ny, nz = 16, 18, 12
    n = nx * ny * nz
    dev = lambda: torch.empty(n, dtype=torch.float64, device="cuda")
    u, v, w, T = dev(), dev(), dev(), dev()
    up, vp, wp, Tp = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(4))
    with mglc_gb300.BuoyancyCavity(nx, ny, nz, rayleigh=1e4, t_hot=0.5, t_cold=-0.5) as c:
        c.initial()
        for call in range(2):
            c.step(30)
            rc = L.mglc_get_macros_device(c.handle, None, u.data_ptr(), v.data_ptr(),
                                          w.data_ptr(), T.data_ptr())
            assert rc == 0
            ref_u, ref_t = c.check()
            got_u, got_t = _noalloc(L, n, u, v, w, T, up, vp, wp, Tp, 1, None)
            np.testing.assert_allclose(got_u, ref_u, rtol=1e-9)
            np.testing.assert_allclose(got_t, ref_t, rtol=1e-9)


@pytest.mark.gpu
def test_noalloc_residual_many_blocks_thermal():
    """64^3 cells = 64 tiles of 4096: the final warp's strided loop over the
    tile partials runs more than once.  Compared with check() on the same
    fields and with a torch FP64 reduction of the same formula."""
    import torch
    import mglc_gb300
    B.build()
    L = capi.lib()
    nx = ny = nz = 64
    n = nx * ny * nz
    assert n > 32 * 4096
    dev = lambda: torch.empty(n, dtype=torch.float64, device="cuda")
    u, v, w, T = dev(), dev(), dev(), dev()
    up, vp, wp, Tp = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(4))
    with mglc_gb300.BuoyancyCavity(nx, ny, nz, rayleigh=1e5, t_hot=0.5, t_cold=-0.5) as c:
        c.initial()
        for call in range(2):
            c.step(40)
            rc = L.mglc_get_macros_device(c.handle, None, u.data_ptr(), v.data_ptr(),
                                          w.data_ptr(), T.data_ptr())
            assert rc == 0
            old = [t.clone() for t in (up, vp, wp, Tp)]
            ref_u, ref_t = c.check()
            got_u, got_t = _noalloc(L, n, u, v, w, T, up, vp, wp, Tp, 1, None)
            np.testing.assert_allclose(got_u, ref_u, rtol=1e-9)
            np.testing.assert_allclose(got_t, ref_t, rtol=1e-9)
            num = ((u - old[0]) ** 2 + (v - old[1]) ** 2 + (w - old[2]) ** 2).sum()
            t_u = (torch.sqrt(num) / torch.sqrt((u * u + v * v + w * w).sum())).item()
            t_t = ((T - old[3]).abs().sum() / T.abs().sum()).item()
            np.testing.assert_allclose(got_u, t_u, rtol=1e-9)
            np.testing.assert_allclose(got_t, t_t, rtol=1e-9)
            assert torch.equal(Tp, T)


@pytest.mark.gpu
def test_noalloc_residual_zero_field_is_numeric_error():
    """A zero velocity field makes errorU 0/0: reported as MGLC_ERR_NUMERIC,
    and the next call on valid fields succeeds."""
    import torch
    B.build()
    L = capi.lib()
    n = 5000
    z = lambda: torch.zeros(n, dtype=torch.float64, device="cuda")
    u, v, w, up, vp, wp = (z() for _ in range(6))
    eu, et = ctypes.c_double(), ctypes.c_double()
    buf = ctypes.create_string_buffer(256)
    rc = L.mglc_residual_noalloc(n, u.data_ptr(), v.data_ptr(), w.data_ptr(), None,
                                 up.data_ptr(), vp.data_ptr(), wp.data_ptr(), None, 0, None,
                                 ctypes.byref(eu), ctypes.byref(et), buf, 256)
    assert rc == 5 and b"not finite" in buf.value and not np.isfinite(eu.value)
    u.fill_(0.5)
    got, _ = _noalloc(L, n, u, v, w, None, up, vp, wp, None, 0, None)
    assert got == pytest.approx(1.0, rel=1e-12)
