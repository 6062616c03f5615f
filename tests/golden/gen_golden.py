"""Generate golden fixtures by executing the MGLC reference's own Fortran source.

Run in a checkout that has the reference tree (default ``/root/reference``):

    python tests/golden/gen_golden.py [--ref PATH]

For each case the reference's module and hot-path subroutines are translated
statement by statement by ``fortran_exec`` and called in the order of the
reference's main loop, on one rank (every MPI exchange is a no-op, every
``MPI_Allreduce`` a copy).  The outputs are written as ``*.npz`` next to this
script.  The test suite checks the C oracle against these files bit for bit,
which pins the oracle to the reference's own statements.

Arrays are stored in numpy with the Fortran index order reversed:
``f(0:18,1:nx,1:ny,1:nz)`` becomes shape ``(nz, ny, nx, 19)``.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from fortran_exec import FArr, Program, preprocess  # noqa: E402

LID_DIR = "MPI/Lid_driven_cavity/fortran/3d/mpi_3d_blocked"
PART_DIR = "MPI/Micro_particles/fortran/case4/mpi_particle"
THERMAL_FILE = "MPI/Buoyancy_driven_cavity/fortran/3d/bouyancy3d_mpi.F90"
LID2D_DIR = "MPI/Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked"
SHEAR_DIR = "MPI/Micro_particles/fortran/case1/mpi_complete"


def _mpi_single_rank(ndim=3):
    dims = FArr([(0, ndim - 1)], np.int64, 1)
    coords = FArr([(0, ndim - 1)], np.int64, 0)
    return {"rank": 0, "rank3d": 0, "num_process": 1, "dims": dims, "coords": coords,
            "periods": FArr([(0, ndim - 1)], np.int64, 0)}


def _interior(arr: FArr):
    """Drop a one-cell halo on the three spatial axes (first numpy axes)."""
    a = arr.numpy()
    return a


def lid_case(ref, nx, ny, nz, reynolds, nsteps, check_every, u0=0.1):
    p = Program()
    p.overrides = {"total_nx": nx, "total_ny": ny, "total_nz": nz, "reynolds": float(reynolds),
                   "u0": float(u0), **_mpi_single_rank()}
    mod = preprocess(open(os.path.join(ref, LID_DIR, "commondata.f90")).read(), p.defines)
    p.load_module(mod)
    p.ns.update({"nx": nx, "ny": ny, "nz": nz})
    for fn in ("initial.f90", "collision.f90", "streaming.f90", "bounce_back.f90", "macro.f90",
               "check.f90"):
        p.load_subroutines(preprocess(open(os.path.join(ref, LID_DIR, fn)).read(), p.defines))
    names = ["initial", "collision", "streaming", "bounceback", "macro", "check"]
    p.build(names)
    p.call("initial")
    ns = p.ns
    out = {"nx": nx, "ny": ny, "nz": nz, "reynolds": float(reynolds), "u0": float(u0),
           "tauf": ns["tauf"], "snu": ns["snu"], "sq": ns["sq"], "nsteps": nsteps,
           "check_every": check_every,
           "f0": ns["f"].numpy(), "rho0": ns["rho"].numpy(), "u_init": ns["u"].numpy()}
    errs = []
    # main.f90:85-102 (message_passing_sendrecv is a no-op on one rank)
    for itc in range(1, nsteps + 1):
        ns["itc"] = itc
        p.call("collision")
        p.call("streaming")
        p.call("bounceback")
        p.call("macro")
        if itc == 1:
            out["f_step1"] = ns["f"].numpy()
        if check_every and itc % check_every == 0:
            p.call("check")
            errs.append(ns["erroru"])
    out.update(f=ns["f"].numpy(), rho=ns["rho"].numpy(), u=ns["u"].numpy(), v=ns["v"].numpy(),
               w=ns["w"].numpy(), erroru=np.array(errs))
    assert not np.isnan(out["f"]).any(), "NaN in f: a halo value was read"
    return out


def thermal_case(ref, nx, ny, nz, rayleigh, prandtl, mach, ekman, thot, tcold, tref, nsteps,
                 check_every, variant="cavity"):
    p = Program()
    p.overrides = {"total_nx": nx, "total_ny": ny, "total_nz": nz, "rayleigh": float(rayleigh),
                   "prandtl": float(prandtl), "mach": float(mach), "ekman": float(ekman),
                   "thot": float(thot), "tcold": float(tcold), "tref": float(tref),
                   **_mpi_single_rank()}
    undef = set()
    if variant == "rb":  # Rayleigh-Benard walls: const-T plates, adiabatic side walls
        undef = {"benchmarkCavity", "LeftRightWallsConstT", "TopBottomPlatesAdiabatic"}
        p.defines |= {"RBconvection", "LeftRightWallsAdiabatic", "TopBottomPlatesConstT"}
    src = preprocess(open(os.path.join(ref, THERMAL_FILE)).read(), p.defines, undef)
    p.load_module(src)
    p.ns.update({"nx": nx, "ny": ny, "nz": nz})
    p.load_subroutines(src)
    names = ["initial", "collision", "streaming", "bounceback", "macro", "collisionT",
             "streamingT", "bouncebackT", "macroT", "check"]
    names = [n.lower() for n in names]
    p.build(names)
    p.call("initial")
    ns = p.ns
    out = {"nx": nx, "ny": ny, "nz": nz, "rayleigh": float(rayleigh), "prandtl": float(prandtl),
           "mach": float(mach), "ekman": float(ekman), "thot": float(thot),
           "tcold": float(tcold), "tref": float(tref), "nsteps": nsteps,
           "check_every": check_every, "variant": variant,
           "tauf": ns["tauf"], "paraa": ns["paraa"], "gbeta": ns["gbeta"],
           "omegaratating": ns["omegaratating"],
           "f0": ns["f"].numpy(), "g0": ns["g"].numpy(), "t_init": ns["t"].numpy()}
    eu, et = [], []
    # bouyancy3d_mpi.F90:222-249
    for itc in range(1, nsteps + 1):
        ns["itc"] = itc
        p.call("collision")
        p.call("streaming")
        p.call("bounceback")
        p.call("collisiont")
        p.call("streamingt")
        p.call("bouncebackt")
        p.call("macro")
        p.call("macrot")
        if itc == 1:
            out["f_step1"] = ns["f"].numpy()
            out["g_step1"] = ns["g"].numpy()
        if check_every and itc % check_every == 0:
            p.call("check")
            eu.append(ns["erroru"])
            et.append(ns["errort"])
    out.update(f=ns["f"].numpy(), g=ns["g"].numpy(), rho=ns["rho"].numpy(), u=ns["u"].numpy(),
               v=ns["v"].numpy(), w=ns["w"].numpy(), T=ns["t"].numpy(), Fx=ns["fx"].numpy(),
               Fy=ns["fy"].numpy(), Fz=ns["fz"].numpy(), erroru=np.array(eu),
               errort=np.array(et))
    assert not np.isnan(out["f"]).any() and not np.isnan(out["g"]).any()
    return out


def lid2d_case(ref, nx, ny, reynolds, nsteps, check_every, u0=0.1):
    """D2Q9 MRT lid-driven cavity on one rank (2d_revised/mpi_blocked,
    main.f90:69-89 order; message_passing is a no-op on one rank)."""
    p = Program()
    p.overrides = {"total_nx": nx, "total_ny": ny, "reynolds": float(reynolds), "u0": float(u0),
                   "rank": 0, "rank2d": 0, "num_process": 1, "comm2d": 0,
                   "dims": FArr([(0, 1)], np.int64, 1), "coords": FArr([(0, 1)], np.int64, 0),
                   "periods": FArr([(0, 1)], np.int64, 0)}
    src = open(os.path.join(ref, LID2D_DIR, "commondata.f90")).read()
    src = src.replace("data periods/2*.false./", "")  # overridden; MPI topology only
    p.load_module(preprocess(src, p.defines))
    p.ns.update({"nx": nx, "ny": ny})
    for fn in ("initial.f90", "evolution.f90", "bounceback.f90"):
        p.load_subroutines(preprocess(open(os.path.join(ref, LID2D_DIR, fn)).read(), p.defines))
    names = ["initial", "collision", "streaming", "bounceback", "macro", "check"]
    p.build(names)
    p.call("initial")
    ns = p.ns
    out = {"nx": nx, "ny": ny, "reynolds": float(reynolds), "u0": float(u0),
           "tauf": ns["tauf"], "snu": ns["snu"], "sq": ns["sq"], "nsteps": nsteps,
           "check_every": check_every, "f0": ns["f"].numpy(), "u_init": ns["u"].numpy()}
    errs = []
    for itc in range(1, nsteps + 1):
        ns["itc"] = itc
        p.call("collision")
        p.call("streaming")
        p.call("bounceback")
        p.call("macro")
        if itc == 1:
            out["f_step1"] = ns["f"].numpy()
        if check_every and itc % check_every == 0:
            p.call("check")
            errs.append(ns["erroru"])
    out.update(f=ns["f"].numpy(), rho=ns["rho"].numpy(), u=ns["u"].numpy(), v=ns["v"].numpy(),
               erroru=np.array(errs))
    assert not np.isnan(out["f"]).any(), "NaN in f: a halo value was read"
    return out


def shear2d_case(ref, nx, ny, radius0, xc, yc, nsteps, frame="stationaryFrame",
                 interp="quadratic", u0=None, uwall=None):
    """case1: one circle carried through a shear flow between walls moving at
    -/+Uwall, periodic in x, on one rank (main.F90:36-72 order).  The centre
    (initial.F90:59-60) is replaced by (xc, yc) for the smaller grid."""
    p = Program()
    p.defines |= {frame, interp}
    ov = {"total_nx": nx, "total_ny": ny, "radius0": float(radius0), "rank": 0, "rank2d": 0,
          "num_process": 1, "comm2d": 0,
          "dims": FArr([(0, 1)], np.int64, 1), "coords": FArr([(0, 1)], np.int64, 0),
          "periods": FArr([(0, 1)], np.int64, 0)}
    if u0 is not None:
        ov["u0"] = float(u0)
    if uwall is not None:
        ov["uwall"] = float(uwall)
    p.overrides = ov
    src = open(os.path.join(ref, SHEAR_DIR, "commondata.F90")).read()
    src = src.replace("data periods/.true., .false./", "")  # overridden; MPI topology only
    p.load_module(preprocess(src, p.defines))
    p.ns.update({"nx": nx, "ny": ny, "i_start_global": 0, "j_start_global": 0})
    ini = open(os.path.join(ref, SHEAR_DIR, "initial.F90")).read()
    lit = lambda x: repr(float(x)) + "d0"  # plain decimals (no exponent) for these centres
    ini = ini.replace("xCenter(1) = 30.0d0", "xCenter(1) = " + lit(xc))
    ini = ini.replace("yCenter(1) = 54.0d0", "yCenter(1) = " + lit(yc))
    for text in (open(os.path.join(ref, SHEAR_DIR, "freeall.F90")).read(), ini,
                 *(open(os.path.join(ref, SHEAR_DIR, fn)).read() for fn in
                   ("fluid.F90", "particle_bounceback.F90", "particle_force.F90",
                    "particle_update.F90"))):
        p.load_subroutines(preprocess(text, p.defines))
    names = ["allocate_all", "initial", "collision", "streaming", "bounceback",
             "bounceback_particle", "calq", "macro", "calforce", "updatecenter"]
    p.build(names)
    p.call("allocate_all")
    p.call("initial")
    ns = p.ns
    out = {"nx": nx, "ny": ny, "radius0": float(radius0), "nsteps": nsteps, "frame": frame,
           "interp": interp, "tauf": ns["tauf"], "rhosolid": ns["rhosolid"], "u0": ns["u0"],
           "uwall": ns["uwall"], "xc0": np.array([[float(xc), float(yc)]])}
    for itc in range(nsteps):
        p.call("collision")
        p.call("streaming")
        p.call("bounceback")
        p.call("bounceback_particle")
        p.call("macro")
        p.call("calforce")
        ns["itc"] = ns["itc"] + 1
        p.call("updatecenter")
    f = ns["f"].numpy()            # (ny+6, nx+6, 9) with lower bound -2
    out.update(f=f[3:3 + ny, 3:3 + nx, :], rho=ns["rho"].numpy(), u=ns["u"].numpy(),
               v=ns["v"].numpy(), obst=ns["obst"].numpy()[1:1 + ny, 1:1 + nx],
               xc=np.stack([ns["xcenter"].numpy(), ns["ycenter"].numpy()], axis=1),
               uc=np.stack([ns["uc"].numpy(), ns["vc"].numpy()], axis=1),
               force=np.stack([ns["walltotalforcex"].numpy(), ns["walltotalforcey"].numpy()], axis=1),
               torque=ns["totaltorque"].numpy(), rho_avg=ns["rhoavg"])
    assert not np.isnan(out["f"]).any()
    return out


def particle2d_case(ref, nx, ny, radius0, gravity, rnd, nsteps):
    """case4 (D2Q9 moving circles) on one rank, main.F90:35-73 order.

    The particle centres come from initial.F90:59-72 with random_number
    returning the values in ``rnd`` (the reference seeds gfortran's generator,
    which is not reproducible here)."""
    p = Program()
    p.overrides = {"total_nx": nx, "total_ny": ny, "cnummax": 2, "radius0": float(radius0),
                   "gravity": float(gravity), "rank": 0, "num_process": 1, "comm2d": 0,
                   "dims": FArr([(0, 1)], np.int64, 1), "coords": FArr([(0, 1)], np.int64, 0),
                   "periods": FArr([(0, 1)], np.int64, 0)}
    mod = preprocess(open(os.path.join(ref, PART_DIR, "commondata.F90")).read(), p.defines)
    p.load_module(mod)
    p.ns.update({"nx": nx, "ny": ny, "i_start_global": 0, "j_start_global": 0})
    for fn in ("freeall.F90", "initial.F90", "fluid.F90", "particle_bounceback.F90",
               "particle_force.F90", "particle_update.F90", "message_particle.F90"):
        p.load_subroutines(preprocess(open(os.path.join(ref, PART_DIR, fn)).read(), p.defines))
    names = ["allocate_all", "initial", "collision", "streaming", "bounceback",
             "bounceback_particle", "calq", "macro", "calforce", "updatecenter",
             "update_particle_mask"]
    p.build(names)
    p.random_values = list(rnd)
    p.call("allocate_all")
    p.call("initial")
    ns = p.ns
    interior = lambda a, lo: a.numpy()[(slice(1 - lo[1], 1 - lo[1] + ny), slice(1 - lo[0], 1 - lo[0] + nx))]
    out = {"nx": nx, "ny": ny, "radius0": float(radius0), "gravity": float(gravity),
           "nsteps": nsteps, "tauf": ns["tauf"], "rhosolid": ns["rhosolid"],
           "xc0": np.stack([ns["xcenter"].numpy(), ns["ycenter"].numpy()], axis=1)}
    for itc in range(nsteps):
        p.call("collision")
        p.call("streaming")
        p.call("bounceback")
        p.call("bounceback_particle")
        p.call("macro")
        p.call("calforce")
        ns["itc"] = ns["itc"] + 1
        p.call("updatecenter")
    f = ns["f"].numpy()            # (ny+6, nx+6, 9) with lower bound -2
    fp = ns["f_post"].numpy()      # (ny+4, nx+4, 9) with lower bound -1
    out.update(f=f[3:3 + ny, 3:3 + nx, :], f_post=fp[2:2 + ny, 2:2 + nx, :],
               rho=ns["rho"].numpy(), u=ns["u"].numpy(), v=ns["v"].numpy(),
               obst=ns["obst"].numpy()[1:1 + ny, 1:1 + nx],
               xc=np.stack([ns["xcenter"].numpy(), ns["ycenter"].numpy()], axis=1),
               uc=np.stack([ns["uc"].numpy(), ns["vc"].numpy()], axis=1),
               omega=ns["rationalomega"].numpy(),
               force=np.stack([ns["walltotalforcex"].numpy(), ns["walltotalforcey"].numpy()], axis=1),
               torque=ns["totaltorque"].numpy(), rho_avg=ns["rhoavg"])
    assert not np.isnan(out["f"]).any()
    return out


CASES = {
    # case4 moving circles: two particles settling, mask updates and refills
    "particle2d_80x50": lambda ref: particle2d_case(ref, 80, 50, 6.0, 0.04,
                                                    [0.513, 0.47, 0.421, 0.552], nsteps=30),
    # D2Q9 lid cavity: non-square grid, Re for tau ~ 0.6 and 1000 (tau ~ 0.52)
    "lid2d_9x7": lambda ref: lid2d_case(ref, 9, 7, reynolds=30.0, nsteps=40, check_every=10),
    "lid2d_12x10_re1000": lambda ref: lid2d_case(ref, 12, 10, reynolds=1000.0, nsteps=25,
                                                 check_every=5),
    # case1 circle in shear flow: the shipped build (stationary frame, quadratic
    # IBB), linear IBB/refill with a faster carrier (more refills), moving frame
    "shear2d_64x40_sq": lambda ref: shear2d_case(ref, 64, 40, 6.25, 24.0, 20.6, nsteps=40),
    "shear2d_56x36_sl": lambda ref: shear2d_case(ref, 56, 36, 5.5, 20.0, 17.3, nsteps=40,
                                                 interp="linear", u0=0.05),
    "shear2d_48x32_mq": lambda ref: shear2d_case(ref, 48, 32, 5.0, 18.0, 15.7, nsteps=30,
                                                 frame="movingFrame"),
    # lid: non-cubic grid to catch axis mix-ups; Re chosen for tau ~ 0.6
    "lid_7x6x5": lambda ref: lid_case(ref, 7, 6, 5, reynolds=21.0, nsteps=12, check_every=4),
    "lid_6x6x6_re400": lambda ref: lid_case(ref, 6, 6, 6, reynolds=400.0, nsteps=6,
                                            check_every=3),
    # thermal as shipped (Thot=1, Tcold=0, Coriolis on via Ekman=1e-3)
    "thermal_6x7x5_ref": lambda ref: thermal_case(ref, 6, 7, 5, 1e4, 0.71, 0.1, 1e-3, 1.0, 0.0,
                                                  0.0, nsteps=8, check_every=4),
    # benchmark-style walls T=+-0.5 and no rotation
    "thermal_5x6x7_pm": lambda ref: thermal_case(ref, 5, 6, 7, 1e5, 0.71, 0.1, float("inf"), 0.5,
                                                 -0.5, 0.0, nsteps=8, check_every=4),
    # Rayleigh-Benard wall variant (const-T plates in z)
    "thermal_6x5x6_rb": lambda ref: thermal_case(ref, 6, 5, 6, 1e4, 0.71, 0.1, 1e-3, 1.0, 0.0,
                                                 0.0, nsteps=6, check_every=3, variant="rb"),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    for name, fn in CASES.items():
        if a.only and a.only != name:
            continue
        t0 = time.time()
        out = fn(a.ref)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in out.items()})
        print(f"{name}: {time.time() - t0:.1f}s -> {os.path.basename(path)}")


if __name__ == "__main__":
    main()
