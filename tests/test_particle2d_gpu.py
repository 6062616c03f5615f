"""The D2Q9 case4 particle step on the GPU against the reference's own
statements: the fixture executed from the reference's Fortran (30 steps, two
settling circles, mask updates and refills) must come out bit for bit, and so
must longer runs of the oracle's literal 2-D mode (both q methods)."""
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


def test_matches_reference_statement_fixture_bitwise(mg):
    d = np.load(os.path.join(GOLD, "particle2d_80x50.npz"))
    with mg.ParticleFlow2D(int(d["nx"]), int(d["ny"]), d["xc0"], float(d["radius0"]),
                           tauf=float(d["tauf"]), rho_solid=float(d["rhosolid"]),
                           gravity=float(d["gravity"])) as c:
        c.initial()
        c.step(int(d["nsteps"]))
        f = c.get_f()
        rho, u, v = c.macro()
        st = c.state()
        m = c.mask()
    assert np.array_equal(f, d["f"])
    for got, key in ((rho, "rho"), (u, "u"), (v, "v")):
        assert np.array_equal(got, d[key]), key
    assert np.array_equal((m >= 0).astype(np.int32), d["obst"])
    assert np.array_equal(st["xc"][:, :2], d["xc"]) and np.array_equal(st["uc"][:, :2], d["uc"])
    assert np.array_equal(st["omega"][:, 2], d["omega"])
    assert np.array_equal(st["force"][:, :2], d["force"]) and np.array_equal(st["torque"][:, 2], d["torque"])


@pytest.mark.parametrize("qmode", [0, 1])
def test_matches_oracle_2d_bitwise(mg, qmode):
    nx, ny, R, g = 90, 120, 7.0, 0.02
    centers = np.array([[24.3, 80.7], [47.9, 95.2], [70.1, 78.4], [35.6, 50.2]])
    o = O.ParticleOracle(np.c_[centers, np.zeros(len(centers))], dim=2, nx=nx, ny=ny, nz=1, tauf=0.7,
                         rho_solid=1.05, radius=R, gravity=(0.0, -g, 0.0), qmode=qmode)
    assert o.step(150) == 0
    r = o.get()
    with mg.ParticleFlow2D(nx, ny, centers, R, tauf=0.7, rho_solid=1.05, gravity=g,
                           q_bisection=qmode == 0) as c:
        c.initial()
        c.step(150)
        f = c.get_f()
        rho, u, v = c.macro()
        st = c.state()
        m = c.mask()
    assert np.array_equal(f, r["f"][0])
    assert np.array_equal(rho, r["rho"][0]) and np.array_equal(u, r["u"][0]) and np.array_equal(v, r["v"][0])
    assert np.array_equal((m >= 0).astype(np.int32), r["obst"][0])
    assert np.array_equal(st["xc"], r["xc"]) and np.array_equal(st["uc"], r["uc"])
    assert np.array_equal(st["omega"], r["om"])
    assert np.array_equal(st["force"], r["force"]) and np.array_equal(st["torque"], r["torque"])
    # the circles settle under gravity and some nodes were refilled on the way
    assert (st["uc"][:, 1] < 0).all()


def test_wall_penetration_is_reported(mg):
    with mg.ParticleFlow2D(40, 40, [[20.0, 7.5]], 6.0, gravity=0.5) as c:
        c.initial()
        with pytest.raises(mg.MglcError) as e:
            c.step(200)
        assert e.value.code == 7


def test_circle_outside_the_box_is_rejected(mg):
    with pytest.raises(mg.MglcError):
        mg.ParticleFlow2D(40, 40, [[3.0, 20.0]], 6.0)


def _seq_sum(x, keep):
    s = 0.0
    for v, k in zip(x.tolist(), keep.tolist()):
        if k:
            s = s + v
    return s


def _gpu_seq_sum(x, keep):
    import ctypes

    from mglc_gb300 import capi
    x = np.ascontiguousarray(x, dtype=np.float64)
    keep = np.ascontiguousarray(keep, dtype=np.int32)
    s, n = ctypes.c_double(), ctypes.c_longlong()
    capi.check(None, capi.lib().mglc_sequential_sum(x.ctypes.data, keep.ctypes.data, x.size,
                                                     ctypes.byref(s), ctypes.byref(n)))
    return s.value, n.value


def _addends(kind, n, rng):
    if kind == "near_one":  # densities: the 2-D particle step's own case
        return 1.0 + 1e-3 * (rng.random(n) - 0.5)
    if kind == "ties":  # few mantissa bits: many exact half-ulp ties
        return np.ldexp(rng.integers(0, 4096, n).astype(np.float64), -12) + 0.5
    if kind == "scales":  # addends across 40 binades, the sum crossing many
        return np.ldexp(rng.random(n), rng.integers(-20, 20, n))
    if kind == "negative":
        x = 3.0 * rng.random(n)
        x[rng.random(n) < 0.002] *= -1.0
        return x
    if kind == "tiny":  # subnormal and zero addends between normal ones
        x = 1.0 + 1e-6 * rng.random(n)
        x[1::2] = 1e-300 * rng.random(x[1::2].size)
        x[::7] = 0.0
        x[::11] = np.ldexp(1.0, -1070)
        return x
    if kind == "specials":
        x = np.ones(n)
        x[::5000] = np.inf
        x[::3333] = np.nan
        return x
    if kind == "signed_zero":
        x = np.full(n, -0.0)
        x[n // 2:] = 1.0
        return x
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["near_one", "ties", "scales", "negative", "tiny", "specials",
                                  "signed_zero"])
@pytest.mark.parametrize("n", [1, 31, 4097, 70001, 320000])
def test_sequential_sum_is_the_loop_order_sum_bitwise(mg, kind, n):
    """The parallel grid sum behind the density averages against the plain
    left-to-right loop, on addends chosen to hit its every path: ties to even,
    binade crossings, negative, subnormal, signed-zero and non-finite addends."""
    rng = np.random.default_rng(n * 7 + len(kind))
    x = _addends(kind, n, rng)
    keep = (rng.random(n) >= 0.1).astype(np.int32)
    got, cnt = _gpu_seq_sum(x, keep)
    want = _seq_sum(x, keep)
    assert cnt == int(keep.sum())
    assert np.array([got]).view(np.int64)[0] == np.array([want]).view(np.int64)[0] or (
        np.isnan(got) and np.isnan(want)), (got, want)


def test_sequential_sum_empty(mg):
    got, cnt = _gpu_seq_sum(np.zeros(0), np.zeros(0, np.int32))
    assert cnt == 0 and got == 0.0 and not np.signbit(got)


@pytest.mark.parametrize("kind", ["near_one", "scales"])
def test_sequential_sum_past_one_scan_tile(mg, kind):
    """4.3 million addends: more than 1024 chunks of 4096, so the chunk scan
    carries its prefix across tiles."""
    n = 4_300_000
    rng = np.random.default_rng(99 + len(kind))
    x = _addends(kind, n, rng)
    keep = (rng.random(n) >= 0.1).astype(np.int32)
    got, cnt = _gpu_seq_sum(x, keep)
    want = _seq_sum(x, keep)
    assert cnt == int(keep.sum())
    assert np.array([got]).view(np.int64)[0] == np.array([want]).view(np.int64)[0], (got, want)
