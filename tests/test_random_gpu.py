"""Seeded randomised parity: lattice shapes, Reynolds/Rayleigh numbers, lid
speed and step counts drawn from a fixed generator, each run against the
oracle (FP64 and FX64 to 1e-10); and a diverging run reported as a numeric
error by check() instead of returning garbage."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(20261204)
LID_CASES = [(int(RNG.integers(3, 40)), int(RNG.integers(3, 40)), int(RNG.integers(3, 40)),
              float(RNG.uniform(50, 2000)), float(RNG.uniform(0.02, 0.15)), int(RNG.integers(1, 200)))
             for _ in range(8)]
TH_CASES = [(int(RNG.integers(4, 30)), int(RNG.integers(4, 30)), int(RNG.integers(4, 30)),
             float(10 ** RNG.uniform(3, 6)), float(RNG.uniform(0.5, 7.0)), int(RNG.integers(1, 150)))
            for _ in range(5)]


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


@pytest.mark.parametrize("case", LID_CASES, ids=[f"{c[0]}x{c[1]}x{c[2]}-Re{c[3]:.0f}" for c in LID_CASES])
@pytest.mark.parametrize("form", ["fp64", "fx64"])
def test_random_lid_cases(mg, case, form):
    nx, ny, nz, re, u0, steps = case
    o = O.LidOracle(nx, ny, nz, re, u0)
    o.run(steps)
    with mg.LidDrivenCavity(nx, ny, nz, reynolds=re, u0=u0, precision=form) as c:
        c.initial()
        c.step(steps)
        f = c.get_f()
        rho, u, v, w = c.macro()
    assert rel_l2(f, o.s.f) <= 1e-12
    assert rel_l2(u, o.s.u) <= 1e-10 and rel_l2(rho, o.s.rho) <= 1e-12


@pytest.mark.parametrize("case", TH_CASES, ids=[f"{c[0]}x{c[1]}x{c[2]}-Ra{c[3]:.0f}" for c in TH_CASES])
@pytest.mark.parametrize("form", ["fp64", "fx64"])
def test_random_thermal_cases(mg, case, form):
    nx, ny, nz, ra, pr, steps = case
    o = O.ThermalOracle(nx, ny, nz, ra, pr, 0.1, 0.0, 0.5, -0.5, 0.0, total_nz=nz)
    o.run(steps)
    with mg.BuoyancyCavity(nx, ny, nz, rayleigh=ra, prandtl=pr, mach=0.1, t_hot=0.5, t_cold=-0.5,
                           precision=form) as c:
        c.initial()
        c.step(steps)
        f, g = c.get_f()
        r = c.macro()
    assert rel_l2(f, o.f) <= 1e-12 and rel_l2(g, o.g) <= 1e-12
    assert rel_l2(r[4], o.T) <= 1e-10


@pytest.mark.parametrize("form", ["fx64", "fp16"])
def test_divergence_is_reported_by_check(mg, form):
    # tau -> 1/2 with a fast lid: these forms leave their range within a few
    # hundred steps (FX64 writes NaN outside its box, FP16 overflows)
    with mg.LidDrivenCavity(16, reynolds=1e7, u0=0.4, precision=form) as c:
        c.initial()
        c.step(600)
        with pytest.raises(mg.MglcError) as e:
            c.check()
    assert e.value.code == 5


@pytest.mark.parametrize("form", ["fp64", "fx64", "fp32", "fp16", "fp16s", "bf16s"])
def test_nonfinite_state_is_reported_by_check(mg, form):
    o = O.LidOracle(12, 11, 10, 200.0, 0.1)
    o.run(5)
    f = o.s.f.copy()
    f[5, 5, 5, 3] = np.nan
    with mg.LidDrivenCavity(12, 11, 10, reynolds=200.0, u0=0.1, precision=form) as c:
        c.load_state(f)
        c.step(3)
        with pytest.raises(mg.MglcError) as e:
            c.check()
    assert e.value.code == 5
