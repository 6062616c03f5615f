"""Python host API over the C-ABI, mirroring the reference's routines.

The reference drives each solve from ``program main`` by calling argument-less
subroutines on module arrays: ``initial()``, then a loop of
``collision(); streaming(); bounceback(); macro()`` and ``check()`` every 2000
steps (MPI/Lid_driven_cavity/fortran/3d/mpi_3d_blocked/main.f90:85-102; the
thermal loop adds ``collisionT/streamingT/bouncebackT/macroT``,
MPI/Buoyancy_driven_cavity/fortran/3d/bouyancy3d_mpi.F90:222-249).  Here one
object holds one solve on the GPU and offers the same verbs:

* ``initial()``            -- the reference initial()
* ``step(n)``              -- n fused time steps (collision .. macro)
* ``macro()``              -- rho, u, v, w (and T) arrays
* ``check()``              -- errorU (and errorT), reference semantics
* ``get_f()`` / ``load_state()`` -- populations in the reference layout

Arrays are numpy, shaped ``(nz, ny, nx)`` for fields and ``(nz, ny, nx, Q)``
for populations, i.e. the Fortran arrays with the index order reversed.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import capi

_P = ctypes.c_void_p


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "need C-contiguous float64"
    return a.ctypes.data


class _Solve:
    Q_G = 0

    def __init__(self):
        self._ctx = _P()

    # -- lifetime --
    def close(self):
        if self._ctx:
            capi.lib().mglc_destroy(self._ctx)
            self._ctx = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        capi.check(self._ctx, rc)

    @property
    def handle(self):
        return self._ctx

    def info(self) -> capi.Info:
        i = capi.Info()
        self._ck(capi.lib().mglc_get_info(self._ctx, ctypes.byref(i)))
        return i

    @property
    def shape(self):
        i = self.info()
        return (i.nz, i.ny, i.nx)

    # -- reference verbs --
    def initial(self):
        self._ck(capi.lib().mglc_initial(self._ctx))
        return self

    def step(self, nsteps: int = 1):
        self._ck(capi.lib().mglc_step(self._ctx, int(nsteps)))
        return self

    def set_stream(self, stream_handle: int | None):
        self._ck(capi.lib().mglc_set_stream(self._ctx, stream_handle))

    def get_f(self):
        nz, ny, nx = self.shape
        f = np.empty((nz, ny, nx, 19))
        g = np.empty((nz, ny, nx, 7)) if self.Q_G else None
        self._ck(capi.lib().mglc_get_f(self._ctx, _ptr(f), _ptr(g)))
        return (f, g) if self.Q_G else f

    def totals(self):
        m, e, h = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._ck(capi.lib().mglc_totals(self._ctx, ctypes.byref(m), ctypes.byref(e), ctypes.byref(h)))
        return m.value, e.value, h.value

    # -- output and checkpoint/restart (the reference's output routines) --
    def _io(self, rc, what, path):
        if rc != capi.MGLC_OK:
            raise capi.MglcError(rc, f"{what} {os.fspath(path)!r} failed")

    def write_tecplot(self, path):
        """output_Tecplot: binary .plt of X Y Z U V W and Pressure (lid) or T."""
        self._io(capi.lib().mglc_write_tecplot(self._ctx, os.fsencode(path)), "Tecplot output", path)

    def write_binary(self, path):
        """output_binary: Fortran unformatted records (lid u, v, rho; heated u, v, w, T)."""
        self._io(capi.lib().mglc_write_binary(self._ctx, os.fsencode(path)), "binary output", path)

    def save_backup(self, path):
        """backupData: Fortran unformatted records u, v, w, (T,) f, (g)."""
        self._io(capi.lib().mglc_backup_save(self._ctx, os.fsencode(path)), "backup", path)

    def load_backup(self, path):
        """The reference's reload: f, g, u, v, w, T from the file, rho = 1."""
        self._io(capi.lib().mglc_backup_load(self._ctx, os.fsencode(path)), "reload", path)
        return self


class NuReMonitor:
    """calNuRe (Buoyancy_driven_cavity/fortran/3d/seq/bouyancy3d.F90:1185-1321):
    feed one (Nu, Re) sample per time unit -- ``sample(cavity)`` takes them
    from a BuoyancyCavity on the device -- and read the running means and the
    stationary / converged flags from the returned status."""

    def __init__(self, flow_reversal=False, flow_reversal_time=0):
        self._m = _P()
        capi.check(None, capi.lib().mglc_nure_create(int(bool(flow_reversal)),
                                                     int(flow_reversal_time), ctypes.byref(self._m)))

    def push(self, nu, re) -> capi.NuReStatus:
        st = capi.NuReStatus()
        capi.check(None, capi.lib().mglc_nure_push(self._m, float(nu), float(re), ctypes.byref(st)))
        return st

    def sample(self, cavity) -> capi.NuReStatus:
        st = capi.NuReStatus()
        capi.check(cavity.handle, capi.lib().mglc_nure_sample(self._m, cavity.handle, ctypes.byref(st)))
        return st

    def close(self):
        if self._m:
            capi.lib().mglc_nure_destroy(self._m)
            self._m = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LidDrivenCavity(_Solve):
    """D3Q19 MRT lid-driven cavity (reference: Lid_driven_cavity/fortran/3d)."""

    def __init__(self, total_nx, total_ny=None, total_nz=None, reynolds=1000.0, u0=0.1,
                 rho0=1.0, top_layer_u0=True, precision="fp64", in_place=False):
        super().__init__()
        self.u0 = float(u0)
        p = capi.LidParams(total_nx, total_ny or total_nx, total_nz or total_nx, float(reynolds),
                           float(rho0), float(u0), int(bool(top_layer_u0)), capi.FORMS[precision],
                           int(bool(in_place)))
        ctx = _P()
        rc = capi.lib().mglc_lid_create(ctypes.byref(p), ctypes.byref(ctx))
        self._ctx = ctx
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_last_error(ctx).decode() if ctx else ""
            self.close()
            raise capi.MglcError(rc, msg)

    def write_profiles(self, uz_path, xw_path):
        """getVelocity: centre-line u(z)/U0 and w(x)/U0 profiles."""
        self._io(capi.lib().mglc_write_profiles(self._ctx, os.fsencode(uz_path), os.fsencode(xw_path),
                                                self.u0), "profiles", uz_path)

    def macro(self):
        nz, ny, nx = self.shape
        rho, u, v, w = (np.empty((nz, ny, nx)) for _ in range(4))
        self._ck(capi.lib().mglc_get_macros(self._ctx, _ptr(rho), _ptr(u), _ptr(v), _ptr(w), None))
        return rho, u, v, w

    def check(self) -> float:
        e = ctypes.c_double()
        self._ck(capi.lib().mglc_check(self._ctx, ctypes.byref(e), None))
        return e.value

    def load_state(self, f, rho=None, u=None, v=None, w=None):
        self._ck(capi.lib().mglc_load_state(self._ctx, _ptr(np.ascontiguousarray(f)), None,
                                            _ptr(rho), _ptr(u), _ptr(v), _ptr(w), None))
        return self


class BuoyancyCavity(_Solve):
    """D3Q19 forced MRT flow + D3Q7 MRT temperature (reference:
    Buoyancy_driven_cavity/fortran/3d/bouyancy3d_mpi.F90)."""

    Q_G = 7

    def __init__(self, total_nx, total_ny=None, total_nz=None, rayleigh=1e5, prandtl=0.71,
                 mach=0.1, t_hot=0.5, t_cold=-0.5, t_ref=0.0, ekman=0.0, bc_y_const_t=True,
                 bc_z_const_t=False, precision="fp64", in_place=False):
        super().__init__()
        p = capi.ThermalParams(total_nx, total_ny or total_nx, total_nz or total_nx,
                               float(rayleigh), float(prandtl), float(mach), float(t_hot),
                               float(t_cold), float(t_ref), float(ekman), int(bool(bc_y_const_t)),
                               int(bool(bc_z_const_t)), capi.FORMS[precision], int(bool(in_place)))
        ctx = _P()
        rc = capi.lib().mglc_thermal_create(ctypes.byref(p), ctypes.byref(ctx))
        self._ctx = ctx
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_last_error(ctx).decode() if ctx else ""
            self.close()
            raise capi.MglcError(rc, msg)

    def macro(self):
        nz, ny, nx = self.shape
        rho, u, v, w, T = (np.empty((nz, ny, nx)) for _ in range(5))
        self._ck(capi.lib().mglc_get_macros(self._ctx, _ptr(rho), _ptr(u), _ptr(v), _ptr(w), _ptr(T)))
        return rho, u, v, w, T

    def check(self):
        eu, et = ctypes.c_double(), ctypes.c_double()
        self._ck(capi.lib().mglc_check(self._ctx, ctypes.byref(eu), ctypes.byref(et)))
        return eu.value, et.value

    def nusselt(self):
        """(Nu_vol, Re_vol, Nu_hot, Nu_cold): calNuRe plus wall Nusselt numbers."""
        vals = [ctypes.c_double() for _ in range(4)]
        self._ck(capi.lib().mglc_nusselt(self._ctx, *[ctypes.byref(v) for v in vals]))
        return tuple(v.value for v in vals)

    def load_state(self, f, g, rho=None, u=None, v=None, w=None, T=None):
        self._ck(capi.lib().mglc_load_state(self._ctx, _ptr(np.ascontiguousarray(f)),
                                            _ptr(np.ascontiguousarray(g)), _ptr(rho), _ptr(u),
                                            _ptr(v), _ptr(w), _ptr(T)))
        return self


class ParticleFlow(_Solve):
    """Moving spheres in a D3Q19 flow (reference: Micro_particles/fortran/case4,
    generalised to 3-D): interpolated bounce-back, momentum-exchange force and
    torque, springs, explicit update and refill."""

    def __init__(self, total_nx, total_ny, total_nz, centers, radius, tauf=0.65, rho0=1.0,
                 rho_solid=1.2, periodic_x=True, gravity=(0.0, 0.0, 0.0),
                 body_force=(0.0, 0.0, 0.0), threshold_wall=2.0, threshold_particle=2.0,
                 spring_scale_wall=1.0, spring_scale_particle=1.0, precision="fp64"):
        super().__init__()
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1, 3))
        self.np = len(c)
        p = capi.ParticleParams(total_nx, total_ny, total_nz, int(bool(periodic_x)), float(tauf),
                                float(rho0), float(rho_solid), float(radius),
                                (ctypes.c_double * 3)(*gravity), (ctypes.c_double * 3)(*body_force),
                                float(threshold_wall), float(threshold_particle),
                                float(spring_scale_wall), float(spring_scale_particle),
                                capi.FORMS[precision])
        ctx = _P()
        rc = capi.lib().mglc_particle_create(ctypes.byref(p), c.ctypes.data, len(c), ctypes.byref(ctx))
        self._ctx = ctx
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_last_error(ctx).decode() if ctx else ""
            self.close()
            raise capi.MglcError(rc, msg)

    def macro(self):
        nz, ny, nx = self.shape
        rho, u, v, w = (np.empty((nz, ny, nx)) for _ in range(4))
        self._ck(capi.lib().mglc_get_macros(self._ctx, _ptr(rho), _ptr(u), _ptr(v), _ptr(w), None))
        return rho, u, v, w

    def state(self):
        out = {k: np.zeros((self.np, 3)) for k in ("xc", "uc", "omega", "force", "torque")}
        self._ck(capi.lib().mglc_particle_state(self._ctx, *[_ptr(out[k]) for k in
                                                             ("xc", "uc", "omega", "force", "torque")]))
        return out

    def mask(self):
        nz, ny, nx = self.shape
        m = np.empty((nz, ny, nx), dtype=np.int32)
        self._ck(capi.lib().mglc_get_mask(self._ctx, m.ctypes.data))
        return m


class ParticleFlow2D(_Solve):
    """D2Q9 moving circles, the reference's own 2-D case4 step
    (Micro_particles/fortran/case4/mpi_particle) with its commondata
    parameters; bitwise the reference's statements.  Arrays are (ny, nx)."""

    def __init__(self, total_nx, total_ny, centers, radius, tauf=0.65, rho0=1.0, rho_solid=1.01,
                 gravity=0.0, threshold_wall=6.0, stiff_wall=0.02, threshold_particle=6.0,
                 stiff_particle=0.08, q_bisection=True):
        super().__init__()
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1, 2))
        self.np = len(c)
        p = capi.Particle2DParams(total_nx, total_ny, float(tauf), float(rho0), float(rho_solid),
                                  float(radius), float(gravity), float(threshold_wall),
                                  float(stiff_wall), float(threshold_particle), float(stiff_particle),
                                  int(bool(q_bisection)))
        ctx = _P()
        rc = capi.lib().mglc_particle2d_create(ctypes.byref(p), c.ctypes.data, len(c), ctypes.byref(ctx))
        self._ctx = ctx
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_last_error(ctx).decode() if ctx else ""
            self.close()
            raise capi.MglcError(rc, msg)

    @property
    def shape2(self):
        i = self.info()
        return (i.ny, i.nx)

    def get_f(self):
        ny, nx = self.shape2
        f = np.empty((ny, nx, 9))
        self._ck(capi.lib().mglc_get_f(self._ctx, _ptr(f), None))
        return f

    def macro(self):
        ny, nx = self.shape2
        rho, u, v = (np.empty((ny, nx)) for _ in range(3))
        self._ck(capi.lib().mglc_get_macros(self._ctx, _ptr(rho), _ptr(u), _ptr(v), None, None))
        return rho, u, v

    def state(self):
        out = {k: np.zeros((self.np, 3)) for k in ("xc", "uc", "omega", "force", "torque")}
        self._ck(capi.lib().mglc_particle_state(self._ctx, *[_ptr(out[k]) for k in
                                                             ("xc", "uc", "omega", "force", "torque")]))
        return out

    def mask(self):
        ny, nx = self.shape2
        m = np.empty((ny, nx), dtype=np.int32)
        self._ck(capi.lib().mglc_get_mask(self._ctx, m.ctypes.data))
        return m


class ShearFlow2D(ParticleFlow2D):
    """D2Q9 circles carried through a shear flow between walls moving at
    -/+uwall, periodic in x: the reference's 2-D case1 step
    (Micro_particles/fortran/case1/mpi_complete) with its commondata
    parameters as defaults; bitwise the reference's statements.  Arrays are
    (ny, nx)."""

    def __init__(self, total_nx, total_ny, centers, radius, tauf=3.0 * (1.0 / 9.0) + 0.5,
                 rho0=1.0, rho_solid=2.0, u0=0.02, uwall=0.1, moving_frame=False, linear=False):
        _Solve.__init__(self)
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1, 2))
        self.np = len(c)
        p = capi.Shear2DParams(total_nx, total_ny, float(tauf), float(rho0), float(rho_solid),
                               float(radius), float(u0), float(uwall), int(bool(moving_frame)),
                               int(bool(linear)))
        ctx = _P()
        rc = capi.lib().mglc_shear2d_create(ctypes.byref(p), c.ctypes.data, len(c), ctypes.byref(ctx))
        self._ctx = ctx
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_last_error(ctx).decode() if ctx else ""
            self.close()
            raise capi.MglcError(rc, msg)


class LidDrivenCavity2D(_Solve):
    """D2Q9 MRT lid-driven cavity, the reference's 2-D code
    (Lid_driven_cavity/fortran/2d/2d_revised/mpi_blocked); bitwise the
    reference's statements, check() included.  Arrays are (ny, nx)."""

    def __init__(self, total_nx, total_ny=None, reynolds=1000.0, u0=0.1, rho0=1.0,
                 precision="fp64"):
        super().__init__()
        self.u0 = float(u0)
        p = capi.Lid2DParams(total_nx, total_ny or total_nx, float(reynolds), float(rho0),
                             float(u0), capi.FORMS[precision])
        ctx = _P()
        rc = capi.lib().mglc_lid2d_create(ctypes.byref(p), ctypes.byref(ctx))
        self._ctx = ctx
        if rc != capi.MGLC_OK:
            msg = capi.lib().mglc_last_error(ctx).decode() if ctx else ""
            self.close()
            raise capi.MglcError(rc, msg)

    @property
    def shape2(self):
        i = self.info()
        return (i.ny, i.nx)

    def get_f(self):
        ny, nx = self.shape2
        f = np.empty((ny, nx, 9))
        self._ck(capi.lib().mglc_get_f(self._ctx, _ptr(f), None))
        return f

    def macro(self):
        ny, nx = self.shape2
        rho, u, v = (np.empty((ny, nx)) for _ in range(3))
        self._ck(capi.lib().mglc_get_macros(self._ctx, _ptr(rho), _ptr(u), _ptr(v), None, None))
        return rho, u, v

    def check(self) -> float:
        e = ctypes.c_double()
        self._ck(capi.lib().mglc_check(self._ctx, ctypes.byref(e), None))
        return e.value

    def load_state(self, f, rho=None, u=None, v=None):
        self._ck(capi.lib().mglc_load_state(self._ctx, _ptr(np.ascontiguousarray(f)), None,
                                            _ptr(rho), _ptr(u), _ptr(v), None, None))
        return self
