import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C-ABI)")
    config.addinivalue_line("markers", "slow: long-running parity case")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU visible")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session", autouse=True)
def _bounds_counter():
    """With MGLC_BOUNDS_CHECK=1 the tests run the diagnostic build whose step
    kernels count every out-of-range element index (and skip the access); the
    session fails at its end unless the count is zero."""
    yield
    if os.environ.get("MGLC_BOUNDS_CHECK") != "1":
        return
    from mglc_gb300 import capi
    if capi._lib is None:  # no test loaded the library
        return
    fn = getattr(capi._lib, "mglc_debug_bounds_hits", None)
    assert fn is not None, "MGLC_BOUNDS_CHECK=1 but the loaded library is not the checked build"
    fn.restype = ctypes.c_ulonglong
    hits = fn()
    assert hits == 0, f"{hits} out-of-range element indices in the step kernels"
