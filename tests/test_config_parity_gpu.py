"""The FP64 plain method against the oracle at the benchmark workloads' own
sizes: the 384^3 lid-driven cavity (Re = 1000, U = 0.1, started at rest) and
the 128^3 differentially heated cavity (Ra = 1e5, Pr = 0.71, Ma = 0.1, walls
at T = +-0.5, no rotation).  Both run on the GPU through the C-ABI and in the
oracle (OpenMP on all host cores) from the same initial state; relative L2
of rho, u, v, w (and T) must stay within 1e-10, over the whole lattice and
separately over the wall cells and the lid layer.

Step counts: 200 of the lid workload's 1000 steps and 2000 of the heated
workload's 20000 (a tenth) by default, which keeps the oracle to about three
minutes on 16 host cores; MGLC_PARITY_LID_STEPS / MGLC_PARITY_THERMAL_STEPS
set other counts (the full 1000 / 20000 take about ten minutes each)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import rel_l2

pytestmark = pytest.mark.gpu

LID_STEPS = int(os.environ.get("MGLC_PARITY_LID_STEPS", "200"))
THERMAL_STEPS = int(os.environ.get("MGLC_PARITY_THERMAL_STEPS", "2000"))
TOL = 1e-10


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _wall_mask(n):
    i = np.arange(n)
    edge = (i == 0) | (i == n - 1)
    return edge[:, None, None] | edge[None, :, None] | edge[None, None, :]


def _compare(got, ref, n, names):
    wall = _wall_mask(n)
    out = {}
    for name, a, b in zip(names, got, ref):
        assert np.isfinite(a).all(), name
        out[name] = (rel_l2(a, b), rel_l2(a[wall], b[wall]), rel_l2(a[-1], b[-1]))
    for name, (whole, walls, top) in out.items():
        assert whole <= TOL, (name, "whole lattice", whole)
        assert walls <= TOL, (name, "wall cells", walls)
        assert top <= TOL, (name, "top layer", top)
    return out


def test_lid_384_cubed_re1000_matches_oracle(mg):
    n = 384
    threads = os.cpu_count() or 1
    with mg.LidDrivenCavity(n, reynolds=1000.0, u0=0.1, top_layer_u0=False) as c:
        c.initial()
        c.step(LID_STEPS)
        got = c.macro()
    o = O.LidOracle(n, n, n, 1000.0, 0.1, top_layer_u0=False)
    o.run(LID_STEPS, nthreads=threads)
    s = o.s
    errs = _compare(got, (s.rho, s.u, s.v, s.w), n, ("rho", "u", "v", "w"))
    assert np.abs(got[1][-1]).max() > 0.01  # the lid has set the top layer moving
    print(f"lid 384^3, {LID_STEPS} steps: " +
          ", ".join(f"{k} {v[0]:.2e}" for k, v in errs.items()))


def test_heated_128_cubed_ra1e5_matches_oracle(mg):
    n = 128
    threads = os.cpu_count() or 1
    with mg.BuoyancyCavity(n, rayleigh=1e5, prandtl=0.71, mach=0.1, t_hot=0.5, t_cold=-0.5,
                           ekman=0.0) as c:
        c.initial()
        c.step(THERMAL_STEPS)
        got = c.macro()
    o = O.ThermalOracle(n, n, n, 1e5, 0.71, 0.1, 0.0, 0.5, -0.5, 0.0)
    o.run(THERMAL_STEPS, nthreads=threads)
    errs = _compare(got, (o.rho, o.u, o.v, o.w, o.T), n, ("rho", "u", "v", "w", "T"))
    assert np.abs(got[3]).max() > 1e-4  # convection has started
    print(f"heated 128^3, {THERMAL_STEPS} steps: " +
          ", ".join(f"{k} {v[0]:.2e}" for k, v in errs.items()))
