"""Host-side output, checkpoint and statistics routines of the library against
the oracle's restatements of the reference's writers (oracle/io_oracle.py):
byte-identical Tecplot streams and Fortran record files, and the calNuRe
state machine step by step.  No GPU needed."""
import ctypes
import os

import numpy as np
import pytest

from mglc_gb300 import capi
from oracle import io_oracle as IO


@pytest.fixture(scope="module")
def lib():
    from mglc_gb300 import build
    build.build()
    return capi.lib()


def _p(a):
    return None if a is None else a.ctypes.data


def _fields(shape, seed):
    rng = np.random.default_rng(seed)
    return [np.ascontiguousarray(rng.standard_normal(shape)) for _ in range(4)]


@pytest.mark.parametrize("thermal", [0, 1])
def test_tecplot_stream_matches_reference_writer(lib, tmp_path, thermal):
    u, v, w, s = _fields((3, 4, 5), 7 + thermal)
    s = s * 0.01 + (0.0 if thermal else 1.0)
    path = str(tmp_path / "out.plt").encode()
    assert lib.mglc_tecplot_write_fields(path, 5, 4, 3, _p(u), _p(v), _p(w), _p(s), thermal) == 0
    got = open(path, "rb").read()
    assert got == IO.tecplot_bytes(u, v, w, s, thermal)


def test_profiles_match_get_velocity(lib, tmp_path):
    u, _, w, _ = _fields((6, 5, 7), 3)
    a, b = str(tmp_path / "uz.dat").encode(), str(tmp_path / "xw.dat").encode()
    assert lib.mglc_profiles_write_fields(a, b, 7, 5, 6, _p(u), _p(w), 0.1) == 0
    uz, xw = IO.profiles(u, w, 0.1)
    assert np.array_equal(np.loadtxt(a.decode()), np.array(uz))
    assert np.array_equal(np.loadtxt(b.decode()), np.array(xw))


@pytest.mark.parametrize("max_sub", [0, 1000, 4096])
@pytest.mark.parametrize("thermal", [0, 1])
def test_backup_records_match_and_round_trip(lib, tmp_path, max_sub, thermal):
    nz, ny, nx = 4, 5, 6
    u, v, w, T = _fields((nz, ny, nx), 11)
    rng = np.random.default_rng(12)
    f = np.ascontiguousarray(rng.random((nz, ny, nx, 19)))
    g = np.ascontiguousarray(rng.random((nz, ny, nx, 7))) if thermal else None
    if not thermal:
        T = None
    path = str(tmp_path / "backup.bin").encode()
    assert lib.mglc_backup_write_fields(path, nx, ny, nz, _p(u), _p(v), _p(w), _p(T), _p(f), _p(g),
                                        max_sub) == 0
    data = open(path, "rb").read()
    assert data == IO.backup_bytes(u, v, w, T, f, g, max_sub or IO.MAX_SUBRECORD)
    recs = IO.read_records(data)
    assert len(recs) == (6 if thermal else 4)
    assert np.array_equal(np.frombuffer(recs[-2 if thermal else -1], "<f8").reshape(f.shape), f)
    out = [np.empty((nz, ny, nx)) for _ in range(4)]
    f2 = np.empty_like(f)
    g2 = np.empty_like(g) if thermal else None
    assert lib.mglc_backup_read_fields(path, nx, ny, nz, _p(out[0]), _p(out[1]), _p(out[2]),
                                       _p(out[3]) if thermal else None, _p(f2), _p(g2)) == 0
    for a, b in zip(out[:3], (u, v, w)):
        assert np.array_equal(a, b)
    assert np.array_equal(f2, f)
    if thermal:
        assert np.array_equal(out[3], T) and np.array_equal(g2, g)


def test_backup_read_rejects_wrong_size_and_truncation(lib, tmp_path):
    nz, ny, nx = 3, 3, 3
    u, v, w, _ = _fields((nz, ny, nx), 5)
    f = np.ascontiguousarray(np.random.default_rng(6).random((nz, ny, nx, 19)))
    path = str(tmp_path / "b.bin").encode()
    assert lib.mglc_backup_write_fields(path, nx, ny, nz, _p(u), _p(v), _p(w), None, _p(f), None, 0) == 0
    big = [np.empty((nz, ny, nx + 1)) for _ in range(3)]
    fb = np.empty((nz, ny, nx + 1, 19))
    assert lib.mglc_backup_read_fields(path, nx + 1, ny, nz, *[_p(a) for a in big], None, _p(fb), None) != 0
    data = open(path, "rb").read()
    cut = str(tmp_path / "cut.bin").encode()
    open(cut, "wb").write(data[:-20])
    ok = [np.empty((nz, ny, nx)) for _ in range(3)]
    assert lib.mglc_backup_read_fields(cut, nx, ny, nz, *[_p(a) for a in ok], None, _p(np.empty_like(f)),
                                       None) != 0
    assert lib.mglc_backup_read_fields(str(tmp_path / "missing.bin").encode(), nx, ny, nz,
                                       *[_p(a) for a in ok], None, _p(np.empty_like(f)), None) != 0


def _series(n, seed, drift):
    """Nu, Re relaxing towards steady values, with noise and an optional
    slow drift (never converging within n samples)."""
    rng = np.random.default_rng(seed)
    t = np.arange(1, n + 1)
    nu = 4.5 + 3.0 * np.exp(-t / 60.0) + 0.02 * rng.standard_normal(n) + drift * t
    re = 120.0 + 80.0 * np.exp(-t / 80.0) + 0.5 * rng.standard_normal(n)
    return nu, re


@pytest.mark.parametrize("fr,frt,drift", [(0, 0, 0.0), (1, 500, 0.0), (0, 0, 2e-3)])
def test_nure_monitor_follows_cal_nu_re(lib, fr, frt, drift):
    import mglc_gb300
    nu, re = _series(1500, 99, drift)
    ref = IO.CalNuRe(fr, frt)
    mon = mglc_gb300.NuReMonitor(bool(fr), frt)
    seen_stat = seen_conv = False
    for a, b in zip(nu, re):
        r = ref.push(float(a), float(b))
        s = mon.push(float(a), float(b))
        assert s.time == r["time"]
        assert s.nu_mean == r["nu_mean"] and s.re_mean == r["re_mean"]
        assert (s.stationary, s.stationary_time, s.converged) == \
            (r["stationary"], r["stationary_time"], r["converged"])
        seen_stat |= bool(s.stationary)
        seen_conv |= bool(s.converged)
    mon.close()
    if drift == 0.0:
        assert seen_stat and seen_conv
    else:  # Nu keeps drifting: the statistics never settle
        assert not seen_conv
