"""The case1 step (circles carried through a shear flow, periodic x) on the
GPU against the reference's own statements: the fixtures executed from the
reference's Fortran (both frames, both interpolation orders) and longer
multi-circle runs of the oracle must come out bit for bit."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _run(mg, nx, ny, centers, radius, steps, **kw):
    with mg.ShearFlow2D(nx, ny, centers, radius, **kw) as c:
        c.initial()
        c.step(steps)
        f = c.get_f()
        rho, u, v = c.macro()
        st = c.state()
        m = c.mask()
    return f, rho, u, v, st, m


@pytest.mark.parametrize("case", ["shear2d_64x40_sq", "shear2d_56x36_sl", "shear2d_48x32_mq"])
def test_matches_reference_statement_fixture_bitwise(mg, case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    f, rho, u, v, st, m = _run(mg, int(d["nx"]), int(d["ny"]), d["xc0"], float(d["radius0"]),
                               int(d["nsteps"]), tauf=float(d["tauf"]),
                               rho_solid=float(d["rhosolid"]), u0=float(d["u0"]),
                               uwall=float(d["uwall"]),
                               moving_frame=str(d["frame"]) == "movingFrame",
                               linear=str(d["interp"]) == "linear")
    assert np.array_equal(f, d["f"])
    for got, key in ((rho, "rho"), (u, "u"), (v, "v")):
        assert np.array_equal(got, d[key]), key
    assert np.array_equal((m >= 0).astype(np.int32), d["obst"])
    assert np.array_equal(st["xc"][:, :2], d["xc"]) and np.array_equal(st["uc"][:, :2], d["uc"])
    assert np.array_equal(st["force"][:, :2], d["force"])
    assert np.array_equal(st["torque"][:, 2], d["torque"])


@pytest.mark.parametrize("moving,linear,steps", [(False, False, 300), (True, True, 200),
                                                 (False, True, 250)])
def test_matches_oracle_bitwise(mg, moving, linear, steps):
    nx, ny, R = 120, 60, 6.5
    centers = np.array([[30.4, 24.7], [74.9, 36.2]])
    kw = dict(u0=0.03, uwall=0.08, moving_frame=moving, linear=linear)
    o = O.ShearOracle(centers, nx, ny, R, **kw)
    assert o.step(steps) == 0
    r = o.get()
    f, rho, u, v, st, m = _run(mg, nx, ny, centers, R, steps, **kw)
    assert np.array_equal(f, r["f"])
    assert np.array_equal(rho, r["rho"]) and np.array_equal(u, r["u"]) and np.array_equal(v, r["v"])
    assert np.array_equal((m >= 0).astype(np.int32), r["obst"])
    assert np.array_equal(st["xc"][:, :2], r["xc"])
    assert np.array_equal(st["force"][:, :2], r["force"])
    assert np.array_equal(st["torque"][:, 2], r["torque"])

