"""Pin the C oracle to the reference: fixtures in tests/golden were produced by
executing the reference's own Fortran statements (tests/golden/gen_golden.py);
the oracle must reproduce them bit for bit."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _cases(prefix):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLD, prefix + "*.npz")))


@pytest.mark.parametrize("case", _cases("lid_"))
def test_lid_oracle_matches_reference_statements(case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    nx, ny, nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
    o = O.LidOracle(nx, ny, nz, float(d["reynolds"]), float(d["u0"]))
    assert (o.tauf, o.snu, o.sq) == (float(d["tauf"]), float(d["snu"]), float(d["sq"]))
    assert np.array_equal(o.s.f, d["f0"])
    errs = []
    for it in range(1, int(d["nsteps"]) + 1):
        o.run(1)
        if it == 1:
            assert np.array_equal(o.s.f, d["f_step1"])
        if it % int(d["check_every"]) == 0:
            errs.append(o.check())
    for k in ("f", "rho", "u", "v", "w"):
        assert np.array_equal(getattr(o.s, k), d[k]), k
    assert np.array_equal(np.array(errs), d["erroru"])


@pytest.mark.parametrize("case", _cases("thermal_"))
def test_thermal_oracle_matches_reference_statements(case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    nx, ny, nz = int(d["nx"]), int(d["ny"]), int(d["nz"])
    ek = float(d["ekman"])
    rb = str(d["variant"]) == "rb"
    o = O.ThermalOracle(nx, ny, nz, float(d["rayleigh"]), float(d["prandtl"]), float(d["mach"]),
                        ek if np.isfinite(ek) else 0.0, float(d["thot"]), float(d["tcold"]),
                        float(d["tref"]), bc_y=0 if rb else 1, bc_z=1 if rb else 0)
    assert o.c.tauf == float(d["tauf"]) and o.c.para_a == float(d["paraa"])
    assert o.c.gbeta == float(d["gbeta"]) and o.c.omega_rot == float(d["omegaratating"])
    assert np.array_equal(o.f, d["f0"]) and np.array_equal(o.g, d["g0"])
    eu, et = [], []
    for it in range(1, int(d["nsteps"]) + 1):
        o.run(1)
        if it == 1:
            assert np.array_equal(o.f, d["f_step1"]) and np.array_equal(o.g, d["g_step1"])
        if it % int(d["check_every"]) == 0:
            a, b = o.check()
            eu.append(a)
            et.append(b)
    for k in ("f", "g", "rho", "u", "v", "w", "T", "Fx", "Fy", "Fz"):
        assert np.array_equal(getattr(o, k), d[k]), k
    assert np.array_equal(np.array(eu), d["erroru"]) and np.array_equal(np.array(et), d["errort"])


def test_oracle_threads_do_not_change_results():
    a = O.LidOracle(9, 8, 7, 50.0, 0.1)
    b = O.LidOracle(9, 8, 7, 50.0, 0.1)
    a.run(5, nthreads=1)
    b.run(5, nthreads=4)
    assert np.array_equal(a.s.f, b.s.f)


@pytest.mark.parametrize("case", _cases("particle2d_"))
def test_particle2d_oracle_matches_reference_statements(case):
    """case4 D2Q9 moving circles: 30 steps with mask updates and refills."""
    d = np.load(os.path.join(GOLD, case + ".npz"))
    xc0 = np.c_[d["xc0"], np.zeros(len(d["xc0"]))]
    o = O.ParticleOracle(xc0, dim=2, nx=int(d["nx"]), ny=int(d["ny"]), nz=1, tauf=float(d["tauf"]),
                         rho_solid=float(d["rhosolid"]), radius=float(d["radius0"]),
                         gravity=(0.0, -float(d["gravity"]), 0.0), qmode=0)
    assert o.step(int(d["nsteps"])) == 0
    g = o.get()
    for k in ("f", "f_post", "rho", "u", "v", "obst"):
        assert np.array_equal(g[k][0], d[k]), k
    assert np.array_equal(g["xc"][:, :2], d["xc"]) and np.array_equal(g["uc"][:, :2], d["uc"])
    assert np.array_equal(g["om"][:, 2], d["omega"])
    assert np.array_equal(g["force"][:, :2], d["force"]) and np.array_equal(g["torque"][:, 2], d["torque"])
    assert g["rho_avg"] == float(d["rho_avg"])


@pytest.mark.parametrize("case", _cases("lid2d_"))
def test_lid2d_oracle_matches_reference_statements(case):
    """D2Q9 MRT lid cavity (2d_revised/mpi_blocked): initial state, step 1,
    the last step and every check() residual, bit for bit."""
    d = np.load(os.path.join(GOLD, case + ".npz"))
    o = O.Lid2DOracle(int(d["nx"]), int(d["ny"]), float(d["reynolds"]), float(d["u0"]))
    assert (o.tauf, o.snu, o.sq) == (float(d["tauf"]), float(d["snu"]), float(d["sq"]))
    assert np.array_equal(o.f, d["f0"]) and np.array_equal(o.u, d["u_init"])
    errs = []
    for it in range(1, int(d["nsteps"]) + 1):
        o.run(1)
        if it == 1:
            assert np.array_equal(o.f, d["f_step1"])
        if it % int(d["check_every"]) == 0:
            errs.append(o.check())
    for k in ("f", "rho", "u", "v"):
        assert np.array_equal(getattr(o, k), d[k]), k
    assert np.array_equal(np.array(errs), d["erroru"])


def test_lid2d_oracle_threads_and_run_checks_agree():
    a = O.Lid2DOracle(33, 21, 400.0, 0.1)
    b = O.Lid2DOracle(33, 21, 400.0, 0.1)
    ea = a.run(60, check_every=20, nthreads=1)
    eb = b.run(60, check_every=20, nthreads=4)
    assert np.array_equal(a.f, b.f) and ea == eb and 0 < ea < 1


def _shear_oracle(d):
    return O.ShearOracle(d["xc0"], int(d["nx"]), int(d["ny"]), float(d["radius0"]),
                         tauf=float(d["tauf"]), rho_solid=float(d["rhosolid"]), u0=float(d["u0"]),
                         uwall=float(d["uwall"]), moving_frame=str(d["frame"]) == "movingFrame",
                         linear=str(d["interp"]) == "linear")


@pytest.mark.parametrize("case", _cases("shear2d_"))
def test_shear2d_oracle_matches_reference_statements(case):
    """case1 circle in shear flow (stationary/moving frame, quadratic/linear):
    populations, fields, mask, centre, velocity, force and torque bit for bit."""
    d = np.load(os.path.join(GOLD, case + ".npz"))
    o = _shear_oracle(d)
    assert o.step(int(d["nsteps"])) == 0
    g = o.get()
    for k in ("f", "rho", "u", "v", "obst", "xc", "uc", "force", "torque"):
        assert np.array_equal(g[k], d[k]), k
    assert g["rho_avg"] == float(d["rho_avg"])
