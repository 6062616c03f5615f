"""Python front end of the solve server (continuous batching, include/mglc.h).

    with SolveServer(hbm_budget_gb=16, precision="fp16") as srv:
        srv.submit("lid", 64, reynolds=400, arrival_s=0.0)
        srv.submit("thermal", 48, rayleigh=1e4, arrival_s=0.05)
        srv.run()
        for r in srv.results(): ...
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi


class SolveServer:
    def __init__(self, hbm_budget_gb=16.0, max_active=64, precision="fp16", steps_per_iteration=200,
                 tol=1e-6, max_steps=50000, autotune=True, keep_results=False, in_place=False):
        p = capi.ServerParams(int(hbm_budget_gb * (1 << 30)), int(max_active), capi.FORMS[precision],
                              int(steps_per_iteration), float(tol), int(max_steps),
                              int(bool(autotune)), int(bool(keep_results)), int(bool(in_place)))
        self._s = ctypes.c_void_p()
        rc = capi.lib().mglc_server_create(ctypes.byref(p), ctypes.byref(self._s))
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_server_last_error(self._s).decode() if self._s else ""
            self.close()
            raise capi.MglcError(rc, msg)
        self.sizes = {}

    def _ck(self, rc):
        if rc != capi.MGLC_OK:
            raise capi.MglcError(rc, capi.lib().mglc_server_last_error(self._s).decode())

    def close(self):
        if self._s:
            capi.lib().mglc_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, kind, n, reynolds=400.0, rayleigh=1e4, arrival_s=0.0) -> int:
        r = capi.Request(capi.KIND_LID if kind == "lid" else capi.KIND_THERMAL, int(n),
                         float(reynolds), float(rayleigh), float(arrival_s))
        rid = ctypes.c_longlong()
        self._ck(capi.lib().mglc_server_submit(self._s, ctypes.byref(r), ctypes.byref(rid)))
        self.sizes[rid.value] = (kind, int(n))
        return rid.value

    def run(self, time_limit_s=3600.0):
        self._ck(capi.lib().mglc_server_run(self._s, float(time_limit_s)))

    def results(self):
        cnt = ctypes.c_int()
        self._ck(capi.lib().mglc_server_results(self._s, None, 0, ctypes.byref(cnt)))
        arr = (capi.RequestResult * max(1, cnt.value))()
        self._ck(capi.lib().mglc_server_results(self._s, arr, cnt.value, ctypes.byref(cnt)))
        return [{k: getattr(arr[q], k) for k, _ in capi.RequestResult._fields_} for q in range(cnt.value)]

    def field(self, rid):
        kind, n = self.sizes[rid]
        planes = 5 if kind == "thermal" else 4
        out = np.empty((planes, n, n, n), dtype=np.float32)
        self._ck(capi.lib().mglc_server_get_field(self._s, rid, out.ctypes.data))
        return out

    def stats(self):
        st = capi.ServerStats()
        self._ck(capi.lib().mglc_server_get_stats(self._s, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in capi.ServerStats._fields_}
