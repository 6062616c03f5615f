"""Parity of the CUDA buoyancy-driven cavity (FP64 drop-in) with the CPU
oracle and with the fixtures executed from the reference's own statements.
Tolerance: FP64 relative L2 <= 1e-10 on rho, u and T."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _make(mg, d):
    ek = float(d["ekman"])
    rb = str(d["variant"]) == "rb"
    return mg.BuoyancyCavity(int(d["nx"]), int(d["ny"]), int(d["nz"]), rayleigh=float(d["rayleigh"]),
                             prandtl=float(d["prandtl"]), mach=float(d["mach"]),
                             t_hot=float(d["thot"]), t_cold=float(d["tcold"]), t_ref=float(d["tref"]),
                             ekman=ek if np.isfinite(ek) else 0.0, bc_y_const_t=not rb,
                             bc_z_const_t=rb)


@pytest.mark.parametrize("case", ["thermal_6x7x5_ref", "thermal_5x6x7_pm", "thermal_6x5x6_rb"])
def test_matches_reference_statement_fixtures(mg, case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    with _make(mg, d) as c:
        c.initial()
        f0, g0 = c.get_f()
        assert np.array_equal(f0, d["f0"]) and np.array_equal(g0, d["g0"])
        c.step(1)
        f1, g1 = c.get_f()
        assert rel_l2(f1, d["f_step1"]) < 1e-14 and rel_l2(g1, d["g_step1"]) < 1e-14
        eu, et = [], []
        for it in range(2, int(d["nsteps"]) + 1):
            c.step(1)
            if it % int(d["check_every"]) == 0:
                pass
        rho, u, v, w, T = c.macro()
        f, g = c.get_f()
    assert rel_l2(f, d["f"]) < 1e-13 and rel_l2(g, d["g"]) < 1e-13
    # early velocities are ~1e-6: compare with a round-off floor (1e-16 of the
    # O(1) populations they are formed from) as well as a relative bound
    for got, key in ((rho, "rho"), (u, "u"), (v, "v"), (w, "w"), (T, "T")):
        np.testing.assert_allclose(got, d[key], rtol=1e-12, atol=1e-15, err_msg=key)


def test_check_matches_reference_semantics(mg):
    d = np.load(os.path.join(GOLD, "thermal_6x7x5_ref.npz"))
    with _make(mg, d) as c:
        c.initial()
        eu, et = [], []
        for it in range(1, int(d["nsteps"]) + 1):
            c.step(1)
            if it % int(d["check_every"]) == 0:
                a, b = c.check()
                eu.append(a)
                et.append(b)
    np.testing.assert_allclose(eu, d["erroru"], rtol=1e-9)
    np.testing.assert_allclose(et, d["errort"], rtol=1e-9)


@pytest.mark.parametrize("ekman", [0.0, 1e-3])
def test_thermal_32_cubed_1000_steps_rel_l2_1e_10(mg, ekman):
    n, steps = 32, 1000
    o = O.ThermalOracle(n, n, n, 1e5, 0.71, 0.1, ekman, 0.5, -0.5, 0.0)
    o.run(steps, nthreads=NT)
    with mg.BuoyancyCavity(n, rayleigh=1e5, prandtl=0.71, mach=0.1, t_hot=0.5, t_cold=-0.5,
                           ekman=ekman) as c:
        c.initial()
        c.step(steps)
        rho, u, v, w, T = c.macro()
    for got, ref, key in ((rho, o.rho, "rho"), (u, o.u, "u"), (v, o.v, "v"), (w, o.w, "w"),
                          (T, o.T, "T")):
        e = rel_l2(got, ref)
        assert e <= 1e-10, (key, e)


def test_macro_of_identical_state_is_bit_exact(mg):
    o = O.ThermalOracle(8, 9, 7, 1e4, 0.71, 0.1, 1e-3, 1.0, 0.0, 0.0)
    o.run(3)
    with mg.BuoyancyCavity(8, 9, 7, rayleigh=1e4, t_hot=1.0, t_cold=0.0, ekman=1e-3) as c:
        c.load_state(o.f, o.g)
        rho, u, v, w, T = c.macro()
    # load_state without macros derives them with F = 0; rho and T do not depend on F
    assert np.array_equal(T, o.T)
    assert np.array_equal(rho, o.rho)


def _nu_numpy(o, axis_y=True):
    """calNuRe (RaNu.F90:13-47) and the wall Nusselt numbers from oracle fields."""
    nz, ny, nx = o.T.shape
    n = nx * ny * nz
    nu_vol = (o.w * o.T).sum() / n * nz / o.c.diffusivity + 1.0
    re_vol = np.sqrt((o.u ** 2 + o.v ** 2 + o.w ** 2).sum() / n) * nz / o.c.viscosity
    dT = o.t_hot - o.t_cold
    T = o.T
    g_hot = (9 * T[:, 0, :] - T[:, 1, :] - 8 * o.t_hot).mean() / 3
    g_cold = (9 * T[:, -1, :] - T[:, -2, :] - 8 * o.t_cold).mean() / 3
    return nu_vol, re_vol, -ny / dT * g_hot, ny / dT * g_cold


def test_nusselt_matches_oracle_fields(mg):
    n, steps = 20, 400
    o = O.ThermalOracle(n, n, n, 1e5, 0.71, 0.1, 0.0, 0.5, -0.5, 0.0)
    o.run(steps, nthreads=NT)
    ref = _nu_numpy(o)
    with mg.BuoyancyCavity(n, rayleigh=1e5, t_hot=0.5, t_cold=-0.5) as c:
        c.initial()
        c.step(steps)
        got = c.nusselt()
    np.testing.assert_allclose(got, ref, rtol=1e-9)
    # heat enters at the hot wall and leaves at the cold wall
    assert got[2] > 1.0 and got[3] > 1.0
