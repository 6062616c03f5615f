"""The in-place (AA-pattern) lid-driven cavity against the two-buffer push
kernel: the arithmetic per cell is the same, so populations, fields and
residuals must agree bit for bit in every form, after odd and even step
counts (an odd count leaves the buffer in the swapped layout, restored on
read), across reloads, and on the 64-bit index path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    from mglc_gb300 import build
    build.build()
    import mglc_gb300
    return mglc_gb300


def _pair(mg, n, form, **kw):
    a = mg.LidDrivenCavity(*n, reynolds=300.0, u0=0.1, precision=form, **kw)
    b = mg.LidDrivenCavity(*n, reynolds=300.0, u0=0.1, precision=form, in_place=True, **kw)
    return a, b


@pytest.mark.parametrize("form", ["fp64", "fx64", "fp32", "fp16", "fp16s", "bf16", "bf16s"])
def test_matches_two_buffer_kernel_bitwise(mg, form):
    a, b = _pair(mg, (33, 35, 37), form)
    with a, b:
        assert b.info().device_bytes < a.info().device_bytes
        for c in (a, b):
            c.initial()
        for steps in (1, 56, 1, 12):  # odd totals leave the swapped layout pending
            a.step(steps)
            b.step(steps)
            assert np.array_equal(a.get_f(), b.get_f())
            for x, y in zip(a.macro(), b.macro()):
                assert np.array_equal(x, y)
            assert a.check() == b.check()


def test_reads_between_steps_do_not_disturb_the_sequence(mg):
    """get_f/macro after an odd step restore the post-stream layout; the next
    step must then start from it (an even step)."""
    a, b = _pair(mg, (24, 20, 18), "fp32")
    with a, b:
        a.initial()
        b.initial()
        for s in range(9):
            a.step(1)
            b.step(1)
            if s % 3 == 0:
                b.macro()
        assert np.array_equal(a.get_f(), b.get_f())


def test_reload_and_totals(mg):
    """The same saved state loaded into both kinds of context continues the same
    (the first step after a load reads the macroscopic fields derived from f)."""
    n = (30, 26, 22)
    with mg.LidDrivenCavity(*n, reynolds=300.0, precision="fp64") as src:
        src.initial()
        src.step(41)
        f = src.get_f()
    a, b = _pair(mg, n, "fp64")
    with a, b:
        a.load_state(f)
        b.load_state(f)
        a.step(33)
        b.step(33)
        assert np.array_equal(a.get_f(), b.get_f())
        assert a.totals() == b.totals()


def test_64bit_index_path(mg):
    """19 x cells >= 2^31 (484^3): in place equals two buffers after 3 steps."""
    n = 484
    a, b = _pair(mg, (n, n, n), "fp16")
    with a, b:
        a.initial()
        b.initial()
        a.step(3)
        b.step(3)
        ra, ua = a.macro()[:2]
        rb, ub = b.macro()[:2]
    assert np.array_equal(ra, rb) and np.array_equal(ua, ub)


@pytest.mark.parametrize("form", ["fp64", "fx64", "fp32", "fp16", "fp16s", "bf16"])
@pytest.mark.parametrize("ekman", [0.0, 1e-3])
def test_heated_cavity_matches_two_buffer_kernel_bitwise(mg, form, ekman):
    """Heated cavity in place (f and g on one buffer each, anti-bounce-back
    walls, carried force, with and without rotation) against two buffers."""
    kw = dict(rayleigh=1e4, t_hot=0.5, t_cold=-0.5, ekman=ekman, precision=form)
    a = mg.BuoyancyCavity(21, 18, 16, **kw)
    b = mg.BuoyancyCavity(21, 18, 16, in_place=True, **kw)
    with a, b:
        assert b.info().device_bytes < a.info().device_bytes
        a.initial()
        b.initial()
        for steps in (1, 30, 3):
            a.step(steps)
            b.step(steps)
            fa, ga = a.get_f()
            fb, gb = b.get_f()
            assert np.array_equal(fa, fb) and np.array_equal(ga, gb)
            for x, y in zip(a.macro(), b.macro()):
                assert np.array_equal(x, y)
        assert a.nusselt() == b.nusselt()


def test_heated_cavity_rayleigh_benard_walls_in_place(mg):
    kw = dict(rayleigh=2e4, t_hot=0.5, t_cold=-0.5, bc_y_const_t=False, bc_z_const_t=True,
              precision="fp32")
    a = mg.BuoyancyCavity(16, 15, 14, **kw)
    b = mg.BuoyancyCavity(16, 15, 14, in_place=True, **kw)
    with a, b:
        a.initial()
        b.initial()
        a.step(25)
        b.step(25)
        assert np.array_equal(a.get_f()[1], b.get_f()[1])
