"""The solve server: continuous batching of cavity solves on one GPU.

Tolerances: a request's fields are bit-identical alone and in a mix (the
per-cell arithmetic does not depend on the other solves or on the tile
shape); a lid request equals the one-solve FP16 context bit for bit; a heated
request agrees with it to 1e-5 (its initial populations are formed in FP32
rather than FP64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _server(mg, **kw):
    args = dict(hbm_budget_gb=2.0, max_active=16, precision="fp16", steps_per_iteration=100,
                tol=1e-12, max_steps=600, autotune=False, keep_results=True)
    args.update(kw)
    return mg.SolveServer(**args)


def test_same_result_alone_and_in_the_mix(mg):
    with _server(mg) as alone:
        rid = alone.submit("lid", 32, reynolds=200.0)
        alone.run()
        ref = alone.field(rid)
        ref_res = alone.results()[0]
    with _server(mg, autotune=True) as mix:
        mix.submit("thermal", 48, rayleigh=2e4, arrival_s=0.0)
        mix.submit("lid", 64, reynolds=800.0, arrival_s=0.0)
        rid2 = mix.submit("lid", 32, reynolds=200.0, arrival_s=0.01)
        mix.submit("thermal", 32, rayleigh=5e3, arrival_s=0.02)
        mix.submit("lid", 48, reynolds=500.0, arrival_s=0.03)
        mix.run()
        got = mix.field(rid2)
        res = {r["id"]: r for r in mix.results()}
        st = mix.stats()
    assert np.array_equal(got, ref)
    assert res[rid2]["steps"] == ref_res["steps"] == 600
    assert st["peak_active"] >= 2 and st["cell_updates"] > 0


def test_lid_request_equals_one_solve_context(mg):
    n, steps = 40, 400
    with _server(mg, max_steps=steps) as srv:
        rid = srv.submit("lid", n, reynolds=300.0)
        srv.run()
        fld = srv.field(rid)
    with mg.LidDrivenCavity(n, reynolds=300.0, u0=0.1, top_layer_u0=False, precision="fp16") as c:
        c.initial()
        c.step(steps)
        rho, u, v, w = c.macro()
    # the server reports FP32 fields formed from the same FP16 state
    np.testing.assert_allclose(fld[1], u, rtol=0, atol=1e-7)
    np.testing.assert_allclose(fld[3], w, rtol=0, atol=1e-7)


@pytest.mark.parametrize("kind", ["lid", "thermal"])
def test_stochastic_rounding_request_matches_one_solve_context(mg, kind):
    """FP16S: the rounding bits come from (cell, step), so a served solve
    stays identical to a one-solve context, in the mix and across iterations."""
    n, steps = 32, 400
    with _server(mg, max_steps=steps, precision="fp16s") as srv:
        other = srv.submit("thermal" if kind == "lid" else "lid", 24, reynolds=200.0, rayleigh=1e4)
        rid = srv.submit(kind, n, reynolds=300.0, rayleigh=1e4)
        srv.run()
        fld = srv.field(rid)
    if kind == "lid":
        c = mg.LidDrivenCavity(n, reynolds=300.0, u0=0.1, top_layer_u0=False, precision="fp16s")
    else:
        c = mg.BuoyancyCavity(n, rayleigh=1e4, prandtl=0.71, mach=0.1, t_hot=0.5, t_cold=-0.5,
                              precision="fp16s")
    with c:
        c.initial()
        c.step(steps)
        u = c.macro()[1]
    np.testing.assert_allclose(fld[1], u, rtol=0, atol=1e-7)


def test_thermal_request_matches_one_solve_context(mg):
    n, steps = 32, 400
    with _server(mg, max_steps=steps) as srv:
        rid = srv.submit("thermal", n, rayleigh=1e4)
        srv.run()
        fld = srv.field(rid)
    with mg.BuoyancyCavity(n, rayleigh=1e4, prandtl=0.71, mach=0.1, t_hot=0.5, t_cold=-0.5,
                           precision="fp16") as c:
        c.initial()
        c.step(steps)
        rho, u, v, w, T = c.macro()
    np.testing.assert_allclose(fld[4], T, rtol=0, atol=1e-5)
    assert np.linalg.norm(fld[3] - w) / np.linalg.norm(w) < 1e-3


def test_admission_respects_the_hbm_budget(mg):
    # a 64^3 FP16 lid solve needs about 23 MiB: a 64 MiB arena holds two
    with _server(mg, hbm_budget_gb=64 / 1024, max_steps=200) as srv:
        for q in range(5):
            srv.submit("lid", 64, reynolds=400.0, arrival_s=0.0)
        srv.run()
        st = srv.stats()
        res = srv.results()
    assert len(res) == 5 and st["peak_active"] == 2
    assert st["peak_device_bytes"] <= 64 * 2 ** 20


def test_late_arrivals_join_running_solves(mg):
    with _server(mg, max_steps=4000) as srv:
        a = srv.submit("lid", 96, reynolds=1000.0, arrival_s=0.0)
        b = srv.submit("lid", 32, reynolds=100.0, arrival_s=0.02)
        srv.run()
        res = {r["id"]: r for r in srv.results()}
    assert res[b]["admit_s"] < res[a]["finish_s"]  # admitted while the first was on the GPU


def test_convergence_retires_early(mg):
    with _server(mg, tol=1e-4, max_steps=50000, steps_per_iteration=200) as srv:
        rid = srv.submit("lid", 24, reynolds=100.0)
        srv.run()
        r = srv.results()[0]
    assert r["converged"] == 1 and r["steps"] < 50000 and r["residual"] < 1e-4


@pytest.mark.parametrize("precision", ["fp16", "fp16s"])
def test_in_place_server_matches_two_buffer_server(mg, precision):
    """AA-pattern serving (one buffer per solve): the same fields as the
    two-buffer server, for lid and heated solves in one mix."""
    out = []
    for in_place in (False, True):
        with _server(mg, max_steps=300, precision=precision, in_place=in_place) as srv:
            ids = [srv.submit("lid", 36, reynolds=400.0), srv.submit("thermal", 28, rayleigh=1e4),
                   srv.submit("lid", 27, reynolds=150.0)]
            srv.run()
            out.append([srv.field(i) for i in ids])
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_in_place_admits_twice_the_solves(mg):
    # a 64^3 FP16 lid solve needs ~23 MiB with two buffers, ~14 MiB in place
    with _server(mg, hbm_budget_gb=64 / 1024, max_steps=200, in_place=True) as srv:
        for q in range(6):
            srv.submit("lid", 64, reynolds=400.0, arrival_s=0.0)
        srv.run()
        st = srv.stats()
    assert st["peak_active"] >= 4
