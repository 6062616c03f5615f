"""FX64 form of the lid-driven cavity: FP64 storage, Q55 fixed-point collision.

It is held to the FP64 drop-in's bar: relative L2 <= 1e-10 against the oracle at
64^3, Re=400, 2000 steps (boundary and lid cells included), and to the
fixtures executed from the reference's own statements."""
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


def test_reports_its_form(mg):
    with mg.LidDrivenCavity(8, reynolds=100.0, u0=0.1, precision="fx64") as c:
        assert c.info().precision == 4


@pytest.mark.parametrize("case", ["lid_7x6x5", "lid_6x6x6_re400"])
def test_matches_reference_statement_fixtures(mg, case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    nx, ny, nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
    with mg.LidDrivenCavity(nx, ny, nz, reynolds=float(d["reynolds"]), u0=float(d["u0"]),
                            precision="fx64") as c:
        c.initial()
        c.step(1)
        assert rel_l2(c.get_f(), d["f_step1"]) < 1e-14
        c.step(int(d["nsteps"]) - 1)
        rho, u, v, w = c.macro()
        assert rel_l2(c.get_f(), d["f"]) < 1e-13
        for got, key in ((rho, "rho"), (u, "u"), (v, "v"), (w, "w")):
            assert rel_l2(got, d[key]) < 1e-12, key


def test_one_step_agrees_with_ieee_fp64(mg):
    o = O.LidOracle(16, 14, 12, 300.0, 0.1)
    o.run(40)
    f40 = o.s.f.copy()
    out = {}
    for form in ("fp64", "fx64"):
        with mg.LidDrivenCavity(16, 14, 12, reynolds=300.0, u0=0.1, precision=form) as c:
            c.load_state(f40)
            c.step(1)
            out[form] = c.get_f()
    assert rel_l2(out["fx64"], out["fp64"]) < 1e-14


def test_first_step_from_stored_macros(mg):
    o = O.LidOracle(12, 10, 9, 300.0, 0.1)
    o.run(5)
    f5 = o.s.f.copy()
    rho5, u5, v5, w5 = o.s.rho.copy(), o.s.u.copy(), o.s.v.copy(), o.s.w.copy()
    o.run(6)
    with mg.LidDrivenCavity(12, 10, 9, reynolds=300.0, u0=0.1, precision="fx64") as c:
        c.load_state(f5, rho5, u5, v5, w5)
        c.step(6)
        assert rel_l2(c.get_f(), o.s.f) < 1e-13


def test_lid_64_cubed_re400_2000_steps_rel_l2_1e_10(mg):
    n, steps = 64, 2000
    o = O.LidOracle(n, n, n, 400.0, 0.1)
    o.run(steps, nthreads=NT)
    with mg.LidDrivenCavity(n, reynolds=400.0, u0=0.1, precision="fx64") as c:
        c.initial()
        c.step(steps)
        rho, u, v, w = c.macro()
    for got, ref, key in ((rho, o.s.rho, "rho"), (u, o.s.u, "u"), (v, o.s.v, "v"), (w, o.s.w, "w")):
        e = rel_l2(got, ref)
        assert e <= 1e-10, (key, e)
    assert rel_l2(u[-1], o.s.u[-1]) <= 1e-10


def test_mass_is_conserved(mg):
    with mg.LidDrivenCavity(24, reynolds=400.0, u0=0.1, precision="fx64") as c:
        c.initial()
        c.step(1)
        m0, _, _ = c.totals()
        c.step(300)
        m1, e1, _ = c.totals()
    assert abs(m1 - m0) / m0 < 1e-12 and e1 > 0


def test_cell_outside_the_range_box_writes_nan(mg):
    """A population of magnitude >= 1 (no physical cavity state has one) turns
    its cell's outputs into NaN instead of wrapping around in fixed point."""
    o = O.LidOracle(10, 9, 8, 200.0, 0.1)
    o.run(3)
    f = o.s.f.copy()
    f[4, 4, 4, 0] = 3.0
    with mg.LidDrivenCavity(10, 9, 8, reynolds=200.0, u0=0.1, precision="fx64") as c:
        c.load_state(f)
        c.step(1)
        g = c.get_f()
    assert np.isnan(g).sum() == 19 and np.isfinite(g[0, 0, 0]).all()


# ------------------------------------------------------------ heated cavity --
def _thermal(mg, d):
    ek = float(d["ekman"])
    rb = str(d["variant"]) == "rb"
    return mg.BuoyancyCavity(int(d["nx"]), int(d["ny"]), int(d["nz"]), rayleigh=float(d["rayleigh"]),
                             prandtl=float(d["prandtl"]), mach=float(d["mach"]),
                             t_hot=float(d["thot"]), t_cold=float(d["tcold"]), t_ref=float(d["tref"]),
                             ekman=ek if np.isfinite(ek) else 0.0, bc_y_const_t=not rb,
                             bc_z_const_t=rb, precision="fx64")


@pytest.mark.parametrize("case", ["thermal_6x7x5_ref", "thermal_5x6x7_pm", "thermal_6x5x6_rb"])
def test_thermal_matches_reference_statement_fixtures(mg, case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    with _thermal(mg, d) as c:
        assert c.info().precision == 4
        c.initial()
        c.step(int(d["nsteps"]))
        rho, u, v, w, T = c.macro()
        f, g = c.get_f()
    assert rel_l2(f, d["f"]) < 1e-13 and rel_l2(g, d["g"]) < 1e-13
    for got, key in ((rho, "rho"), (T, "T")):
        assert rel_l2(got, d[key]) < 1e-12, key
    for got, key in ((u, "u"), (v, "v"), (w, "w")):
        np.testing.assert_allclose(got, d[key], rtol=1e-9, atol=1e-14, err_msg=key)


@pytest.mark.parametrize("ekman", [0.0, 1e-3])
def test_thermal_32_cubed_1000_steps_rel_l2_1e_10(mg, ekman):
    n, steps = 32, 1000
    o = O.ThermalOracle(n, n, n, 1e5, 0.71, 0.1, ekman, 0.5, -0.5, 0.0)
    o.run(steps, nthreads=NT)
    with mg.BuoyancyCavity(n, rayleigh=1e5, prandtl=0.71, mach=0.1, t_hot=0.5, t_cold=-0.5,
                           ekman=ekman, precision="fx64") as c:
        c.initial()
        c.step(steps)
        rho, u, v, w, T = c.macro()
    for got, ref, key in ((rho, o.rho, "rho"), (u, o.u, "u"), (v, o.v, "v"), (w, o.w, "w"),
                          (T, o.T, "T")):
        e = rel_l2(got, ref)
        assert e <= 1e-10, (key, e)


def test_thermal_one_step_agrees_with_ieee_fp64(mg):
    out = {}
    for form in ("fp64", "fx64"):
        with mg.BuoyancyCavity(20, 18, 16, rayleigh=1e5, t_hot=0.5, t_cold=-0.5, precision=form) as c:
            c.initial()
            c.step(60)
            out[form] = c.get_f()
    assert rel_l2(out["fx64"][0], out["fp64"][0]) < 1e-13
    assert rel_l2(out["fx64"][1], out["fp64"][1]) < 1e-13
