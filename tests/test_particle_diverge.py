"""A particle state that diverges is reported, not looped on.

The periodic-x separation of a node from a sphere centre takes one shift by the
period while centres stay inside [0.5, nx + 0.5); the update step reports a
centre, velocity or spin that is not finite, or a centre that moved half the
period or more in one step (status 7, MGLC_ERR_PARTICLE on the GPU path), and
every later kernel leaves the frozen state alone.  The drive is an acceleration
on the particle alone (``gravity`` acts as (rho_s - rho_avg) V g on the
spheres, not on the fluid), so the first failing check is this one.
Only the particle is pushed: nothing here faults or hangs a GPU."""
import math

import numpy as np
import pytest

from oracle import oracle as O

CASE = dict(nx=24, ny=20, nz=20, radius=3.0, tauf=0.65, rho_solid=1.2, periodic_x=1,
            threshold_wall=2.0, threshold_particle=2.0, spring_scale_wall=1e-3,
            spring_scale_particle=1e-3)
CENTER = [[12.3, 10.4, 10.2]]
# (rho_s - rho_avg)/rho_s * g / 2 is the first step's move: 0.5 * (0.2/1.2) * 180 = 15 >= 12
DRIVES = [(180.0, 0.0, 0.0), (math.inf, 0.0, 0.0), (0.0, math.nan, 0.0)]
# a sphere that drifts across the periodic boundary x = nx + 0.5 at a physical speed
CROSS, CROSS_G, CROSS_STEPS = [[24.0, 10.4, 10.2]], (5e-3, 0.0, 0.0), 90


@pytest.mark.parametrize("g", DRIVES, ids=["jump", "inf", "nan"])
def test_oracle_reports_divergence(g):
    o = O.ParticleOracle(np.array(CENTER), dim=3, qmode=1, gravity=g, **CASE)
    assert o.step(3) == 7


def test_oracle_periodic_crossing_is_unchanged():
    """A sphere drifting across the periodic boundary at a physical speed wraps
    once per step and never trips the divergence check."""
    o = O.ParticleOracle(np.array(CROSS), dim=3, qmode=1, gravity=CROSS_G, **CASE)
    assert o.step(CROSS_STEPS) == 0
    x = o.get()["xc"][0, 0]
    assert 0.5 <= x < CASE["nx"] + 0.5


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _flow(mg, g, precision="fp64", centers=CENTER):
    k = CASE
    return mg.ParticleFlow(k["nx"], k["ny"], k["nz"], centers, k["radius"], tauf=k["tauf"],
                           rho_solid=k["rho_solid"], periodic_x=True, gravity=g,
                           threshold_wall=k["threshold_wall"],
                           threshold_particle=k["threshold_particle"],
                           spring_scale_wall=k["spring_scale_wall"],
                           spring_scale_particle=k["spring_scale_particle"], precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("g", DRIVES, ids=["jump", "inf", "nan"])
def test_gpu_reports_divergence_and_freezes(mg, g, precision):
    from mglc_gb300.capi import MglcError
    with _flow(mg, g, precision) as c:
        c.initial()
        with pytest.raises(MglcError) as ei:
            c.step(3)
        assert ei.value.code == 7 and "diverged" in str(ei.value)
        # the state stays frozen at the failing step: further steps change nothing
        f0 = c.get_f()
        with pytest.raises(MglcError):
            c.step(2)
        assert np.array_equal(c.get_f(), f0, equal_nan=True)


@pytest.mark.gpu
def test_gpu_periodic_crossing_matches_oracle(mg):
    """The wrap keeps its old result for physical moves: a sphere crossing the
    periodic boundary stays bit-compatible with the oracle (FP64 1e-10)."""
    o = O.ParticleOracle(np.array(CROSS), dim=3, qmode=1, gravity=CROSS_G, **CASE)
    assert o.step(CROSS_STEPS) == 0
    ref = o.get()
    with _flow(mg, CROSS_G, centers=CROSS) as c:
        c.initial()
        c.step(CROSS_STEPS)
        st = c.state()
    np.testing.assert_allclose(st["xc"], ref["xc"], rtol=0, atol=1e-9)
    assert ref["xc"][0, 0] < 12.0  # it crossed the boundary
