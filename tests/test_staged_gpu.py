"""The lid step with bulk-copy staged loads (k_step_tma.cu) against the
one-thread-per-cell kernel with direct loads: the same arithmetic, so every
population must be bitwise equal.  MGLC_LID_TMA=0 at context creation selects
the direct-load kernel.  Grids cover one and several x segments per row,
partial last segments (x extents 8 cells past a multiple of 128), rows that
are not a multiple of 16 bytes (which take the direct-load kernel either way),
and the 64-bit index path."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMS = ["fp32", "fp16", "fp16s", "bf16", "bf16s"]


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _run(mg, shape, form, steps, staged, reload_every=0):
    old = os.environ.get("MGLC_LID_TMA")
    os.environ["MGLC_LID_TMA"] = "1" if staged else "0"
    try:
        c = mg.LidDrivenCavity(*shape, reynolds=400.0, u0=0.1, top_layer_u0=False,
                               precision=form)
    finally:
        if old is None:
            os.environ.pop("MGLC_LID_TMA")
        else:
            os.environ["MGLC_LID_TMA"] = old
    with c:
        c.initial()
        done = 0
        while done < steps:
            k = min(steps - done, reload_every or steps)
            c.step(k)
            done += k
            if reload_every:
                c.macro()  # reads between steps must not disturb the staged kernel
        return c.get_f()


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("shape", [(48, 20, 16), (136, 9, 7), (264, 5, 6), (40, 7, 3)])
def test_staged_loads_bitwise_equal_direct(mg, form, shape):
    a = _run(mg, shape, form, 37, True)
    b = _run(mg, shape, form, 37, False)
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("form", ["fp16s", "fp32"])
def test_staged_loads_with_reads_between_steps(mg, form):
    a = _run(mg, (64, 24, 20), form, 30, True, reload_every=7)
    b = _run(mg, (64, 24, 20), form, 30, False, reload_every=7)
    assert np.array_equal(a, b)


def test_rows_not_16_byte_multiple_use_direct_loads(mg):
    """nx = 36 FP16 (72-byte rows): the staged kernel does not apply; both
    settings run the direct-load kernel and agree."""
    a = _run(mg, (36, 10, 8), "fp16", 20, True)
    b = _run(mg, (36, 10, 8), "fp16", 20, False)
    assert np.array_equal(a, b)


def test_staged_loads_64bit_index_path(mg):
    """488^3 FP16: 19 * cells >= 2^31, so both kernels index with 64 bits;
    the macroscopic fields after 3 steps are compared on the device."""
    import torch
    from mglc_gb300 import capi
    n = 488
    assert 19 * n ** 3 >= 2 ** 31
    out = []
    for staged in (True, False):
        os.environ["MGLC_LID_TMA"] = "1" if staged else "0"
        try:
            c = mg.LidDrivenCavity(n, reynolds=1000.0, u0=0.1, top_layer_u0=False,
                                   precision="fp16")
        finally:
            os.environ.pop("MGLC_LID_TMA")
        with c:
            c.initial()
            c.step(3)
            f = [torch.empty(n ** 3, dtype=torch.float64, device="cuda") for _ in range(4)]
            rc = capi.lib().mglc_get_macros_device(c.handle, *[t.data_ptr() for t in f], None)
            assert rc == 0
            out.append(f)
        torch.cuda.synchronize()
    for x, y in zip(*out):
        assert torch.equal(x, y)
    assert out[0][1].abs().max().item() > 0.01
