"""ctypes front end of the CPU oracle (``oracle/lbm_oracle.c``).

TEST INFRASTRUCTURE ONLY: the test suite, the smoke check and bench.py's
CPU-baseline leg use this module as the checker.  The product library never
imports it.

Arrays use the reference's Fortran layout (population index fastest,
column-major), held in numpy as C-contiguous arrays of shape
``(nz, ny, nx, Q)`` for ``f(0:Q-1,1:nx,1:ny,1:nz)`` and ``(nz, ny, nx)`` for the
macroscopic fields.  The haloed post-collision arrays have shape
``(nz+2, ny+2, nx+2, Q)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-O2 -ffp-contract=off, OpenMP for the timed baseline)."""
    srcs = [os.path.join(HERE, f) for f in ("lbm_oracle.c", "particle_oracle.c", "lid2d_oracle.c", "shear2d_oracle.c")]
    hdr = os.path.join(HERE, "lbm_oracle.h")
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(x) for x in srcs + [hdr])
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
               "-shared", "-o", LIB, *srcs, "-lm"]
        subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _declare(_lib)
    return _lib


_D = ctypes.c_double
_I = ctypes.c_int
_P = ctypes.POINTER(ctypes.c_double)


class ThConsts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("tauf", "viscosity", "diffusivity", "omega_rot", "para_a", "gbeta",
                 "snu", "sq", "qd", "qnu")]


class ShearParams(ctypes.Structure):
    _fields_ = [("nx", _I), ("ny", _I), ("np", _I), ("moving_frame", _I), ("linear", _I),
                ("tauf", _D), ("rho0", _D), ("rho_solid", _D), ("radius", _D), ("u0", _D),
                ("uwall", _D)]


def _declare(L):
    L.orc_lid_params.argtypes = [_I, _D, _D, _P, _P, _P]
    L.orc_lid_initial.argtypes = [_I, _I, _I, _D, _D, _I, _P, _P, _P, _P, _P]
    L.orc_lid_collision.argtypes = [_I, _I, _I, _D, _D, _P, _P, _P, _P, _P, _P]
    L.orc_lid_streaming.argtypes = [_I, _I, _I, _P, _P]
    L.orc_lid_bounceback.argtypes = [_I, _I, _I, _D, _P, _P, _P]
    L.orc_lid_macro.argtypes = [_I, _I, _I, _P, _P, _P, _P, _P]
    L.orc_lid_check.argtypes = [_I, _I, _I, _P, _P, _P, _P, _P, _P]
    L.orc_lid_check.restype = _D
    L.orc_lid_run.argtypes = [_I, _I, _I, _D, _D, _D, _I, _I, _I] + [_P] * 9
    L.orc_lid_run.restype = _D
    L.orc_lid2d_params.argtypes = [_I, _D, _D, _P, _P, _P]
    L.orc_lid2d_initial.argtypes = [_I, _I, _D, _D, _P, _P, _P, _P]
    L.orc_lid2d_check.argtypes = [_I, _I, _P, _P, _P, _P]
    L.orc_lid2d_check.restype = _D
    L.orc_lid2d_run.argtypes = [_I, _I, _D, _D, _D, _I, _I, _I] + [_P] * 7
    L.orc_lid2d_run.restype = _D
    L.orc_shear_create.argtypes = [ctypes.POINTER(ShearParams), _P]
    L.orc_shear_create.restype = ctypes.c_void_p
    L.orc_shear_step.argtypes = [ctypes.c_void_p, _I]
    L.orc_shear_get.argtypes = [ctypes.c_void_p, _P, _P, _P, _P, ctypes.c_void_p, _P, _P, _P, _P, _P]
    L.orc_shear_destroy.argtypes = [ctypes.c_void_p]
    TP = ctypes.POINTER(ThConsts)
    L.orc_th_params.argtypes = [_I, _D, _D, _D, _D, TP]
    L.orc_th_initial.argtypes = [_I, _I, _I, TP, _D, _D, _I, _I] + [_P] * 7
    L.orc_th_check.argtypes = [_I, _I, _I] + [_P] * 8 + [_P, _P]
    L.orc_th_run.argtypes = [_I, _I, _I, TP, _D, _D, _D, _I, _I, _I, _I] + [_P] * 12
    L.orc_pt_create.argtypes = [ctypes.POINTER(ParticleParams), _P]
    L.orc_pt_create.restype = ctypes.c_void_p
    L.orc_pt_step.argtypes = [ctypes.c_void_p, _I]
    L.orc_pt_step.restype = _I
    _IP = ctypes.POINTER(ctypes.c_int)
    L.orc_pt_get.argtypes = [ctypes.c_void_p, _P, _P, _P, _P, _P, _P, _IP, _P, _P, _P, _P, _P, _P]
    L.orc_pt_destroy.argtypes = [ctypes.c_void_p]


class ParticleParams(ctypes.Structure):
    _fields_ = [("dim", _I), ("nx", _I), ("ny", _I), ("nz", _I), ("periodic_x", _I), ("np", _I),
                ("tauf", _D), ("rho0", _D), ("rho_solid", _D), ("radius", _D),
                ("gravity", _D * 3), ("body_force", _D * 3), ("threshold_wall", _D),
                ("stiff_wall", _D), ("threshold_particle", _D), ("stiff_particle", _D),
                ("spring_scale_wall", _D), ("spring_scale_particle", _D), ("qmode", _I)]


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def lid_params(total_nx: int, reynolds: float, u0: float):
    t, s1, s2 = _D(), _D(), _D()
    lib().orc_lid_params(total_nx, reynolds, u0, ctypes.byref(t), ctypes.byref(s1), ctypes.byref(s2))
    return t.value, s1.value, s2.value


@dataclass
class LidState:
    nx: int
    ny: int
    nz: int
    f: np.ndarray
    f_post: np.ndarray
    rho: np.ndarray
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    up: np.ndarray
    vp: np.ndarray
    wp: np.ndarray


class LidOracle:
    """Reference lid-driven cavity (mpi_3d_blocked on one rank)."""

    def __init__(self, nx, ny, nz, reynolds, u0, rho0=1.0, top_layer_u0=True, total_nx=None):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.u0 = u0
        self.tauf, self.snu, self.sq = lid_params(total_nx or nx, reynolds, u0)
        z = lambda *s: np.zeros(s, dtype=np.float64)
        self.s = LidState(nx, ny, nz, z(nz, ny, nx, 19), z(nz + 2, ny + 2, nx + 2, 19),
                          z(nz, ny, nx), z(nz, ny, nx), z(nz, ny, nx), z(nz, ny, nx),
                          z(nz, ny, nx), z(nz, ny, nx), z(nz, ny, nx))
        s = self.s
        lib().orc_lid_initial(nx, ny, nz, u0, rho0, int(bool(top_layer_u0)), _p(s.f), _p(s.rho),
                              _p(s.u), _p(s.v), _p(s.w))
        self.itc = 0

    def run(self, nsteps: int, check_every: int = 0, nthreads: int = 1) -> float:
        s = self.s
        err = lib().orc_lid_run(self.nx, self.ny, self.nz, self.snu, self.sq, self.u0, nsteps,
                                check_every, nthreads, _p(s.f), _p(s.f_post), _p(s.rho),
                                _p(s.u), _p(s.v), _p(s.w), _p(s.up), _p(s.vp), _p(s.wp))
        self.itc += nsteps
        return err

    def check(self) -> float:
        s = self.s
        return lib().orc_lid_check(self.nx, self.ny, self.nz, _p(s.u), _p(s.v), _p(s.w),
                                   _p(s.up), _p(s.vp), _p(s.wp))


class Lid2DOracle:
    """Reference D2Q9 lid-driven cavity (2d_revised/mpi_blocked on one rank).
    f has shape (ny, nx, 9), f_post (ny+2, nx+2, 9), fields (ny, nx)."""

    def __init__(self, nx, ny, reynolds, u0, rho0=1.0, total_nx=None):
        self.nx, self.ny, self.u0 = nx, ny, u0
        t, s1, s2 = _D(), _D(), _D()
        lib().orc_lid2d_params(total_nx or nx, reynolds, u0, ctypes.byref(t), ctypes.byref(s1),
                               ctypes.byref(s2))
        self.tauf, self.snu, self.sq = t.value, s1.value, s2.value
        z = lambda *s: np.zeros(s, dtype=np.float64)
        self.f, self.f_post = z(ny, nx, 9), z(ny + 2, nx + 2, 9)
        self.rho, self.u, self.v, self.up, self.vp = (z(ny, nx) for _ in range(5))
        lib().orc_lid2d_initial(nx, ny, u0, rho0, _p(self.f), _p(self.rho), _p(self.u),
                                _p(self.v))
        self.itc = 0

    def run(self, nsteps: int, check_every: int = 0, nthreads: int = 1) -> float:
        err = lib().orc_lid2d_run(self.nx, self.ny, self.snu, self.sq, self.u0, nsteps,
                                  check_every, nthreads, _p(self.f), _p(self.f_post),
                                  _p(self.rho), _p(self.u), _p(self.v), _p(self.up), _p(self.vp))
        self.itc += nsteps
        return err

    def check(self) -> float:
        return lib().orc_lid2d_check(self.nx, self.ny, _p(self.u), _p(self.v), _p(self.up),
                                     _p(self.vp))


def th_params(total_nz, rayleigh, prandtl, mach, ekman) -> ThConsts:
    c = ThConsts()
    lib().orc_th_params(total_nz, rayleigh, prandtl, mach, ekman, ctypes.byref(c))
    return c


class ThermalOracle:
    """Reference buoyancy-driven cavity (bouyancy3d_mpi.F90 on one rank)."""

    def __init__(self, nx, ny, nz, rayleigh, prandtl, mach, ekman, t_hot, t_cold, t_ref,
                 bc_y=1, bc_z=0, total_nz=None):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.c = th_params(total_nz or nz, rayleigh, prandtl, mach, ekman)
        self.t_hot, self.t_cold, self.t_ref = t_hot, t_cold, t_ref
        self.bc_y, self.bc_z = bc_y, bc_z
        z = lambda *s: np.zeros(s, dtype=np.float64)
        self.f = z(nz, ny, nx, 19)
        self.f_post = z(nz + 2, ny + 2, nx + 2, 19)
        self.g = z(nz, ny, nx, 7)
        self.g_post = z(nz + 2, ny + 2, nx + 2, 7)
        self.rho, self.u, self.v, self.w, self.T = (z(nz, ny, nx) for _ in range(5))
        self.Fx, self.Fy, self.Fz = (z(nz, ny, nx) for _ in range(3))
        self.up, self.vp, self.wp, self.Tp = (z(nz, ny, nx) for _ in range(4))
        lib().orc_th_initial(nx, ny, nz, ctypes.byref(self.c), t_hot, t_cold, bc_y, bc_z,
                             _p(self.f), _p(self.g), _p(self.rho), _p(self.u), _p(self.v),
                             _p(self.w), _p(self.T))
        self.itc = 0

    def run(self, nsteps: int, nthreads: int = 1):
        lib().orc_th_run(self.nx, self.ny, self.nz, ctypes.byref(self.c), self.t_ref, self.t_hot,
                         self.t_cold, self.bc_y, self.bc_z, nsteps, nthreads, _p(self.f),
                         _p(self.f_post), _p(self.g), _p(self.g_post), _p(self.rho), _p(self.u),
                         _p(self.v), _p(self.w), _p(self.T), _p(self.Fx), _p(self.Fy),
                         _p(self.Fz))
        self.itc += nsteps

    def check(self):
        eu, et = _D(), _D()
        lib().orc_th_check(self.nx, self.ny, self.nz, _p(self.u), _p(self.v), _p(self.w),
                           _p(self.T), _p(self.up), _p(self.vp), _p(self.wp), _p(self.Tp),
                           ctypes.byref(eu), ctypes.byref(et))
        return eu.value, et.value


class ParticleOracle:
    """Moving particles: dim=2 is the literal case4 D2Q9 restatement, dim=3
    the D3Q19 sphere generalisation."""

    def __init__(self, centers, **kw):
        centers = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
        p = ParticleParams()
        defaults = dict(dim=3, nx=16, ny=16, nz=16, periodic_x=0, np=len(centers), tauf=0.65,
                        rho0=1.0, rho_solid=1.2, radius=3.0, gravity=(0.0, 0.0, 0.0),
                        body_force=(0.0, 0.0, 0.0), threshold_wall=6.0, stiff_wall=0.02,
                        threshold_particle=6.0, stiff_particle=0.08, spring_scale_wall=0.0,
                        spring_scale_particle=0.0, qmode=0)
        defaults.update(kw)
        defaults["np"] = len(centers)
        for k, v in defaults.items():
            if k in ("gravity", "body_force"):
                getattr(p, k)[:] = list(v)
            else:
                setattr(p, k, v)
        self.p = p
        self.Q = 9 if p.dim == 2 else 19
        self._s = lib().orc_pt_create(ctypes.byref(p), _p(centers))

    def step(self, n=1) -> int:
        return lib().orc_pt_step(self._s, n)

    def get(self):
        p = self.p
        nz = p.nz if p.dim == 3 else 1
        shp = (nz, p.ny, p.nx)
        out = {k: np.zeros(shp) for k in ("rho", "u", "v", "w")}
        out["f"] = np.zeros(shp + (self.Q,))
        out["f_post"] = np.zeros(shp + (self.Q,))
        out["obst"] = np.zeros(shp, dtype=np.int32)
        for k in ("xc", "uc", "om", "force", "torque"):
            out[k] = np.zeros((p.np, 3))
        ra = ctypes.c_double()
        lib().orc_pt_get(self._s, _p(out["f"]), _p(out["f_post"]), _p(out["rho"]), _p(out["u"]),
                         _p(out["v"]), _p(out["w"]),
                         out["obst"].ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(out["xc"]),
                         _p(out["uc"]), _p(out["om"]), _p(out["force"]), _p(out["torque"]),
                         ctypes.byref(ra))
        out["rho_avg"] = ra.value
        return out

    def __del__(self):
        try:
            lib().orc_pt_destroy(self._s)
        except Exception:
            pass


class ShearOracle:
    """case1 (circles in shear flow, periodic x) on one rank.  Fields (ny, nx),
    f (ny, nx, 9), per-circle vectors (np, 2)."""

    def __init__(self, centers, nx, ny, radius, tauf=3.0 * (1.0 / 9.0) + 0.5, rho0=1.0,
                 rho_solid=2.0, u0=0.02, uwall=0.1, moving_frame=False, linear=False):
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1, 2))
        self.nx, self.ny, self.np = nx, ny, len(c)
        self.p = ShearParams(nx, ny, len(c), int(bool(moving_frame)), int(bool(linear)),
                             float(tauf), float(rho0), float(rho_solid), float(radius), float(u0),
                             float(uwall))
        self.h = lib().orc_shear_create(ctypes.byref(self.p), _p(c))

    def step(self, n=1) -> int:
        return lib().orc_shear_step(self.h, n)

    def get(self):
        nx, ny, k = self.nx, self.ny, max(self.np, 1)
        o = {"f": np.zeros((ny, nx, 9)), "rho": np.zeros((ny, nx)), "u": np.zeros((ny, nx)),
             "v": np.zeros((ny, nx)), "obst": np.zeros((ny, nx), dtype=np.int32),
             "xc": np.zeros((k, 2)), "uc": np.zeros((k, 2)), "force": np.zeros((k, 2)),
             "torque": np.zeros(k)}
        ra = ctypes.c_double()
        lib().orc_shear_get(self.h, _p(o["f"]), _p(o["rho"]), _p(o["u"]), _p(o["v"]),
                            o["obst"].ctypes.data, _p(o["xc"]), _p(o["uc"]), _p(o["force"]),
                            _p(o["torque"]), ctypes.byref(ra))
        o["rho_avg"] = ra.value
        return o

    def __del__(self):
        try:
            lib().orc_shear_destroy(self.h)
        except Exception:
            pass
