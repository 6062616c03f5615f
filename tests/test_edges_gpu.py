"""Edge cases against the oracle: odd and non-cubic lattices (rows that do not
fill a warp, 2-cell-thin directions), the non-periodic particle box and the
particle channel without particles."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


@pytest.mark.parametrize("shape", [(33, 35, 37), (2, 9, 5), (41, 3, 2), (65, 7, 19)])
@pytest.mark.parametrize("form", ["fp64", "fx64"])
def test_lid_odd_shapes_match_oracle(mg, shape, form):
    nx, ny, nz = shape
    o = O.LidOracle(nx, ny, nz, 250.0, 0.1)
    o.run(120)
    with mg.LidDrivenCavity(nx, ny, nz, reynolds=250.0, u0=0.1, precision=form) as c:
        c.initial()
        c.step(120)
        rho, u, v, w = c.macro()
        f = c.get_f()
    assert rel_l2(f, o.s.f) <= 1e-12
    for got, ref in ((rho, o.s.rho), (u, o.s.u), (w, o.s.w)):
        assert rel_l2(got, ref) <= 1e-10


@pytest.mark.parametrize("shape", [(31, 29, 33), (5, 40, 6)])
def test_thermal_odd_shapes_match_oracle(mg, shape):
    nx, ny, nz = shape
    o = O.ThermalOracle(nx, ny, nz, 1e5, 0.71, 0.1, 0.0, 0.5, -0.5, 0.0, total_nz=nz)
    o.run(150)
    with mg.BuoyancyCavity(nx, ny, nz, rayleigh=1e5, prandtl=0.71, mach=0.1, t_hot=0.5,
                           t_cold=-0.5) as c:
        c.initial()
        c.step(150)
        f, g = c.get_f()
        r = c.macro()
    assert rel_l2(f, o.f) <= 1e-12 and rel_l2(g, o.g) <= 1e-12
    assert rel_l2(r[4], o.T) <= 1e-10


KW = dict(tauf=0.65, rho_solid=1.2, gravity=(0.0, 0.0, -2e-5), threshold_wall=2.0,
          threshold_particle=2.0, spring_scale_wall=1e-3, spring_scale_particle=1e-3)


def _pair(mg, centers, periodic, body, shape=(36, 26, 24), steps=50):
    nx, ny, nz = shape
    o = O.ParticleOracle(np.array(centers).reshape(-1, 3), dim=3, qmode=1, nx=nx, ny=ny, nz=nz,
                         radius=3.5, periodic_x=int(periodic), body_force=body, **KW)
    assert o.step(steps) == 0
    r = o.get()
    with mg.ParticleFlow(nx, ny, nz, np.array(centers).reshape(-1, 3), 3.5, periodic_x=periodic,
                         body_force=body, **KW) as c:
        c.initial()
        c.step(steps)
        return r, c.get_f(), c.state(), c.mask()


def test_particles_in_a_closed_box_match_oracle(mg):
    r, f, st, m = _pair(mg, [[10.2, 12.6, 11.4], [24.7, 13.1, 12.2]], False, (0.0, 0.0, 0.0))
    fluid = r["obst"] == 0
    assert np.array_equal(m < 0, fluid)
    assert rel_l2(f[fluid], r["f"][fluid]) <= 1e-10
    assert rel_l2(st["uc"], r["uc"]) <= 1e-9 and rel_l2(st["force"], r["force"]) <= 1e-9


def test_channel_without_particles_matches_oracle(mg):
    nx, ny, nz = 20, 18, 16
    o = O.ParticleOracle(np.zeros((0, 3)), dim=3, qmode=1, nx=nx, ny=ny, nz=nz, radius=3.5,
                         periodic_x=1, body_force=(1e-5, 0.0, 0.0), **KW)
    assert o.step(80) == 0
    r = o.get()
    with mg.ParticleFlow(nx, ny, nz, np.zeros((0, 3)), 3.5, periodic_x=True,
                         body_force=(1e-5, 0.0, 0.0), **KW) as c:
        c.initial()
        c.step(80)
        f = c.get_f()
        rho, u, v, w = c.macro()
    assert rel_l2(f, r["f"]) <= 1e-12
    # body-force driven channel: flow along +x, symmetric about the duct centre
    assert (u[1:-1, 1:-1, :] > 0).all()
    np.testing.assert_allclose(u, u[:, ::-1, :], rtol=0, atol=1e-15)
