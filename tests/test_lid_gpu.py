"""Parity of the CUDA lid-driven cavity (FP64 drop-in) with the CPU oracle and
with the fixtures executed from the reference's own statements.

Tolerances: FP64 relative L2 <= 1e-10 after the stated step count (the
reference-parity bar); the initial state and macro() of an identical state are
bit-exact."""
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


def test_initial_state_is_bit_exact(mg):
    o = O.LidOracle(9, 7, 6, 100.0, 0.1)
    with mg.LidDrivenCavity(9, 7, 6, reynolds=100.0, u0=0.1) as c:
        c.initial()
        assert np.array_equal(c.get_f(), o.s.f)
        rho, u, v, w = c.macro()
        assert np.array_equal(u, o.s.u) and np.array_equal(rho, o.s.rho)


@pytest.mark.parametrize("case", ["lid_7x6x5", "lid_6x6x6_re400"])
def test_matches_reference_statement_fixtures(mg, case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    nx, ny, nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
    with mg.LidDrivenCavity(nx, ny, nz, reynolds=float(d["reynolds"]), u0=float(d["u0"])) as c:
        c.initial()
        c.step(1)
        assert rel_l2(c.get_f(), d["f_step1"]) < 1e-14
        c.step(int(d["nsteps"]) - 1)
        # residual semantics: test_check_matches_reference_semantics; fields here
        rho, u, v, w = c.macro()
        assert rel_l2(c.get_f(), d["f"]) < 1e-13
        for got, key in ((rho, "rho"), (u, "u"), (v, "v"), (w, "w")):
            np.testing.assert_allclose(got, d[key], rtol=1e-12, atol=1e-15, err_msg=key)


def test_check_matches_reference_semantics(mg):
    d = np.load(os.path.join(GOLD, "lid_7x6x5.npz"))
    with mg.LidDrivenCavity(7, 6, 5, reynolds=float(d["reynolds"]), u0=float(d["u0"])) as c:
        c.initial()
        errs = []
        for it in range(1, int(d["nsteps"]) + 1):
            c.step(1)
            if it % int(d["check_every"]) == 0:
                errs.append(c.check())
    np.testing.assert_allclose(errs, d["erroru"], rtol=1e-9)


def test_macro_of_identical_state_is_bit_exact(mg):
    o = O.LidOracle(10, 9, 8, 200.0, 0.1)
    o.run(7)
    with mg.LidDrivenCavity(10, 9, 8, reynolds=200.0, u0=0.1) as c:
        c.load_state(o.s.f)
        assert np.array_equal(c.get_f(), o.s.f)
        rho, u, v, w = c.macro()
        for got, ref in ((rho, o.s.rho), (u, o.s.u), (v, o.s.v), (w, o.s.w)):
            assert np.array_equal(got, ref)


def test_load_state_with_macros_continues_like_the_reference(mg):
    o = O.LidOracle(12, 10, 9, 300.0, 0.1)
    o.run(5)
    f5 = o.s.f.copy()
    rho5, u5, v5, w5 = o.s.rho.copy(), o.s.u.copy(), o.s.v.copy(), o.s.w.copy()
    o.run(6)
    with mg.LidDrivenCavity(12, 10, 9, reynolds=300.0, u0=0.1) as c:
        c.load_state(f5, rho5, u5, v5, w5)
        c.step(6)
        assert rel_l2(c.get_f(), o.s.f) < 1e-13


def test_lid_64_cubed_re400_2000_steps_rel_l2_1e_10(mg):
    """The reference-parity case: 64^3, Re=400, U=0.1, 2000 steps, FP64."""
    n, steps = 64, 2000
    o = O.LidOracle(n, n, n, 400.0, 0.1)
    o.run(steps, nthreads=NT)
    with mg.LidDrivenCavity(n, reynolds=400.0, u0=0.1) as c:
        c.initial()
        c.step(steps)
        rho, u, v, w = c.macro()
        for got, ref, key in ((rho, o.s.rho, "rho"), (u, o.s.u, "u"), (v, o.s.v, "v"),
                              (w, o.s.w, "w")):
            e = rel_l2(got, ref)
            assert e <= 1e-10, (key, e)
        # boundary and lid cells included: check the top layer separately too
        assert rel_l2(u[-1], o.s.u[-1]) <= 1e-10


def test_mass_is_conserved(mg):
    with mg.LidDrivenCavity(24, reynolds=400.0, u0=0.1) as c:
        c.initial()
        c.step(1)
        m0, _, _ = c.totals()
        c.step(300)
        m1, e1, _ = c.totals()
    assert abs(m1 - m0) / m0 < 1e-12 and e1 > 0


def test_y_mirror_symmetry(mg):
    """The lid moves along x, so the flow is mirror-symmetric about y = ny/2."""
    with mg.LidDrivenCavity(16, 16, 16, reynolds=100.0, u0=0.1) as c:
        c.initial()
        c.step(200)
        rho, u, v, w = c.macro()
    np.testing.assert_allclose(u, u[:, ::-1, :], rtol=0, atol=1e-13)
    np.testing.assert_allclose(v, -v[:, ::-1, :], rtol=0, atol=1e-13)


def test_step_before_initial_is_a_state_error(mg):
    c = mg.LidDrivenCavity(8, reynolds=100.0)
    with pytest.raises(mg.MglcError) as ei:
        c.step(1)
    assert ei.value.code == 4
    c.close()
