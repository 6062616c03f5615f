"""The D2Q9 lid-driven cavity on the GPU against the reference's own
statements (2d_revised/mpi_blocked): the fixtures executed from the
reference's Fortran and longer runs of the oracle, including the reference's
own 201 x 201, Re = 1000 configuration, must come out bit for bit -- fields,
populations and every check() residual."""
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


@pytest.mark.parametrize("case", ["lid2d_9x7", "lid2d_12x10_re1000"])
def test_matches_reference_statement_fixture_bitwise(mg, case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    with mg.LidDrivenCavity2D(int(d["nx"]), int(d["ny"]), reynolds=float(d["reynolds"]),
                              u0=float(d["u0"])) as c:
        i = c.info()
        assert (i.tauf, i.snu, i.sq) == (float(d["tauf"]), float(d["snu"]), float(d["sq"]))
        c.initial()
        assert np.array_equal(c.get_f(), d["f0"])
        assert np.array_equal(c.macro()[1], d["u_init"])
        errs = []
        for it in range(1, int(d["nsteps"]) + 1):
            c.step(1)
            if it == 1:
                assert np.array_equal(c.get_f(), d["f_step1"])
            if it % int(d["check_every"]) == 0:
                errs.append(c.check())
        f = c.get_f()
        rho, u, v = c.macro()
    assert np.array_equal(f, d["f"])
    for got, key in ((rho, "rho"), (u, "u"), (v, "v")):
        assert np.array_equal(got, d[key]), key
    assert np.array_equal(np.array(errs), d["erroru"])


@pytest.mark.parametrize("nx,ny,re,steps,every", [(201, 201, 1000.0, 2000, 500),
                                                  (96, 40, 100.0, 700, 350),
                                                  (17, 130, 400.0, 400, 100)])
def test_matches_oracle_bitwise(mg, nx, ny, re, steps, every):
    o = O.Lid2DOracle(nx, ny, re, 0.1)
    oerr = []
    for _ in range(steps // every):
        oerr.append(o.run(every, check_every=every, nthreads=8))
    with mg.LidDrivenCavity2D(nx, ny, reynolds=re, u0=0.1) as c:
        c.initial()
        gerr = []
        for _ in range(steps // every):
            c.step(every)
            gerr.append(c.check())
        f = c.get_f()
        rho, u, v = c.macro()
        assert c.info().itc == steps
    assert np.array_equal(f, o.f)
    assert np.array_equal(rho, o.rho) and np.array_equal(u, o.u) and np.array_equal(v, o.v)
    assert gerr == oerr


def test_reload_continues_bitwise(mg):
    """mglc_load_state with f alone (fields derived, as macro() would) and
    with f + rho,u,v both continue exactly like the uninterrupted run."""
    nx, ny = 48, 36
    with mg.LidDrivenCavity2D(nx, ny, reynolds=300.0) as a:
        a.initial()
        a.step(150)
        f = a.get_f()
        rho, u, v = a.macro()
        a.step(100)
        ref = a.get_f()
    for fields in (None, (rho, u, v)):
        with mg.LidDrivenCavity2D(nx, ny, reynolds=300.0) as b:
            if fields is None:
                b.load_state(f)
            else:
                b.load_state(f, *fields)
            b.step(100)
            assert np.array_equal(b.get_f(), ref)


def test_mass_is_conserved_and_state_is_finite(mg):
    with mg.LidDrivenCavity2D(64, 64, reynolds=1000.0) as c:
        c.initial()
        m0, e0, _ = c.totals()
        c.step(3000)
        m1, e1, _ = c.totals()
    assert abs(m1 - m0) < 1e-9 * m0 and np.isfinite(e1) and e1 > 0
