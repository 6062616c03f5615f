"""ctypes binding of ``libmglc_gb300.so`` (the C-ABI in include/mglc.h).

This is the Python side of the same ABI a Fortran host binds through
iso_c_binding.  Loading fails loudly when the library has not been built:
there is no CPU fallback anywhere in the product.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# MGLC_BOUNDS_CHECK=1 selects the bounds-checked diagnostic build (mglc_gb300/build.py)
LIB_PATH = os.path.join(HERE, "_build_checked" if os.environ.get("MGLC_BOUNDS_CHECK") == "1"
                        else "_build", "libmglc_gb300.so")

MGLC_OK = 0
ERRORS = {1: "MGLC_ERR_INVALID", 2: "MGLC_ERR_CUDA", 3: "MGLC_ERR_NOMEM", 4: "MGLC_ERR_STATE",
          5: "MGLC_ERR_NUMERIC", 6: "MGLC_ERR_UNSUPPORTED", 7: "MGLC_ERR_PARTICLE"}
FORMS = {"fp64": 0, "fp32": 1, "fp16": 2, "bf16": 3, "fx64": 4, "fp16s": 5, "bf16s": 6}
KIND_LID, KIND_THERMAL, KIND_PARTICLE = 1, 2, 3

_D, _I, _LL = ctypes.c_double, ctypes.c_int, ctypes.c_longlong
_DP = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


class LidParams(ctypes.Structure):
    _fields_ = [("total_nx", _I), ("total_ny", _I), ("total_nz", _I), ("reynolds", _D),
                ("rho0", _D), ("u0", _D), ("top_layer_u0", _I), ("precision", _I),
                ("in_place", _I)]


class ThermalParams(ctypes.Structure):
    _fields_ = [("total_nx", _I), ("total_ny", _I), ("total_nz", _I), ("rayleigh", _D),
                ("prandtl", _D), ("mach", _D), ("t_hot", _D), ("t_cold", _D), ("t_ref", _D),
                ("ekman", _D), ("bc_y_const_t", _I), ("bc_z_const_t", _I), ("precision", _I),
                ("in_place", _I)]


class ParticleParams(ctypes.Structure):
    _fields_ = [("total_nx", _I), ("total_ny", _I), ("total_nz", _I), ("periodic_x", _I),
                ("tauf", _D), ("rho0", _D), ("rho_solid", _D), ("radius", _D),
                ("gravity", _D * 3), ("body_force", _D * 3), ("threshold_wall", _D),
                ("threshold_particle", _D), ("spring_scale_wall", _D),
                ("spring_scale_particle", _D), ("precision", _I)]


class Info(ctypes.Structure):
    _fields_ = [("kind", _I), ("precision", _I), ("nx", _I), ("ny", _I), ("nz", _I),
                ("itc", _LL), ("tauf", _D), ("snu", _D), ("sq", _D), ("viscosity", _D),
                ("diffusivity", _D), ("para_a", _D), ("gbeta", _D), ("omega_rot", _D),
                ("bytes_per_cell_step", _D), ("device_bytes", _LL)]


class ServerParams(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", _LL), ("max_active", _I), ("precision", _I),
                ("steps_per_iteration", _I), ("tol", _D), ("max_steps", _LL), ("autotune", _I),
                ("keep_results", _I), ("in_place", _I)]


class Request(ctypes.Structure):
    _fields_ = [("kind", _I), ("n", _I), ("reynolds", _D), ("rayleigh", _D), ("arrival_s", _D)]


class RequestResult(ctypes.Structure):
    _fields_ = [("id", _LL), ("kind", _I), ("n", _I), ("steps", _LL), ("residual", _D),
                ("arrival_s", _D), ("admit_s", _D), ("finish_s", _D), ("converged", _I)]


class ServerStats(ctypes.Structure):
    _fields_ = [("iterations", _LL), ("steps_total", _LL), ("cell_updates", _LL), ("wall_s", _D),
                ("busy_s", _D), ("tile_threads", _I), ("tile_rows", _I), ("ctas_per_sm", _I),
                ("peak_device_bytes", _LL), ("peak_active", _I)]


class Particle2DParams(ctypes.Structure):
    _fields_ = [("total_nx", _I), ("total_ny", _I), ("tauf", _D), ("rho0", _D), ("rho_solid", _D),
                ("radius", _D), ("gravity", _D), ("threshold_wall", _D), ("stiff_wall", _D),
                ("threshold_particle", _D), ("stiff_particle", _D), ("q_bisection", _I)]


class Shear2DParams(ctypes.Structure):
    _fields_ = [("total_nx", _I), ("total_ny", _I), ("tauf", _D), ("rho0", _D), ("rho_solid", _D),
                ("radius", _D), ("u0", _D), ("uwall", _D), ("moving_frame", _I), ("linear", _I)]


class Lid2DParams(ctypes.Structure):
    _fields_ = [("total_nx", _I), ("total_ny", _I), ("reynolds", _D), ("rho0", _D), ("u0", _D),
                ("precision", _I)]


class NuReStatus(ctypes.Structure):
    _fields_ = [("time", _I), ("nu", _D), ("re", _D), ("nu_mean", _D), ("re_mean", _D),
                ("stationary", _I), ("stationary_time", _I), ("converged", _I),
                ("nu_half_change", _D), ("re_half_change", _D), ("nu_mean_change", _D),
                ("re_mean_change", _D)]


# (name, argtypes, restype) of every exported symbol; tests check that the
# library exports all of them
SIGNATURES = {
    "mglc_lid_create": ([ctypes.POINTER(LidParams), ctypes.POINTER(_VP)], _I),
    "mglc_thermal_create": ([ctypes.POINTER(ThermalParams), ctypes.POINTER(_VP)], _I),
    "mglc_particle_create": ([ctypes.POINTER(ParticleParams), _VP, _I, ctypes.POINTER(_VP)], _I),
    "mglc_particle_state": ([_VP, _VP, _VP, _VP, _VP, _VP], _I),
    "mglc_particle2d_create": ([ctypes.POINTER(Particle2DParams), _VP, _I, ctypes.POINTER(_VP)], _I),
    "mglc_lid2d_create": ([ctypes.POINTER(Lid2DParams), ctypes.POINTER(_VP)], _I),
    "mglc_shear2d_create": ([ctypes.POINTER(Shear2DParams), _VP, _I, ctypes.POINTER(_VP)], _I),
    "mglc_get_mask": ([_VP, _VP], _I),
    "mglc_destroy": ([_VP], None),
    "mglc_last_error": ([_VP], ctypes.c_char_p),
    "mglc_set_stream": ([_VP, _VP], _I),
    "mglc_get_info": ([_VP, ctypes.POINTER(Info)], _I),
    "mglc_initial": ([_VP], _I),
    "mglc_load_state": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP], _I),
    "mglc_get_f": ([_VP, _VP, _VP], _I),
    "mglc_step": ([_VP, _I], _I),
    "mglc_get_macros": ([_VP, _VP, _VP, _VP, _VP, _VP], _I),
    "mglc_get_macros_device": ([_VP, _VP, _VP, _VP, _VP, _VP], _I),
    "mglc_check": ([_VP, _DP, _DP], _I),
    "mglc_totals": ([_VP, _DP, _DP, _DP], _I),
    "mglc_nusselt": ([_VP, _DP, _DP, _DP, _DP], _I),
    "mglc_server_create": ([ctypes.POINTER(ServerParams), ctypes.POINTER(_VP)], _I),
    "mglc_server_destroy": ([_VP], None),
    "mglc_server_last_error": ([_VP], ctypes.c_char_p),
    "mglc_server_submit": ([_VP, ctypes.POINTER(Request), ctypes.POINTER(_LL)], _I),
    "mglc_server_run": ([_VP, _D], _I),
    "mglc_server_results": ([_VP, _VP, _I, ctypes.POINTER(_I)], _I),
    "mglc_server_get_field": ([_VP, _LL, _VP], _I),
    "mglc_server_get_stats": ([_VP, ctypes.POINTER(ServerStats)], _I),
    "mglc_residual_noalloc": ([_LL, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _I, _VP, _DP, _DP,
                               ctypes.c_char_p, _I], _I),
    "mglc_write_tecplot": ([_VP, ctypes.c_char_p], _I),
    "mglc_tecplot_write_fields": ([ctypes.c_char_p, _I, _I, _I, _VP, _VP, _VP, _VP, _I], _I),
    "mglc_write_profiles": ([_VP, ctypes.c_char_p, ctypes.c_char_p, _D], _I),
    "mglc_profiles_write_fields": ([ctypes.c_char_p, ctypes.c_char_p, _I, _I, _I, _VP, _VP, _D], _I),
    "mglc_write_binary": ([_VP, ctypes.c_char_p], _I),
    "mglc_backup_save": ([_VP, ctypes.c_char_p], _I),
    "mglc_backup_load": ([_VP, ctypes.c_char_p], _I),
    "mglc_backup_write_fields": ([ctypes.c_char_p, _I, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP, _LL], _I),
    "mglc_backup_read_fields": ([ctypes.c_char_p, _I, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP], _I),
    "mglc_nure_create": ([_I, _I, ctypes.POINTER(_VP)], _I),
    "mglc_nure_destroy": ([_VP], None),
    "mglc_nure_push": ([_VP, _D, _D, ctypes.POINTER(NuReStatus)], _I),
    "mglc_nure_sample": ([_VP, _VP, ctypes.POINTER(NuReStatus)], _I),
    "mglc_sequential_sum": ([_VP, _VP, _I, _DP, ctypes.POINTER(_LL)], _I),
}

_lib = None


class MglcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib():
    """Load the built library (raises if it is missing: no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with mglc_gb300.build.build() "
                               "(or __graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (argt, rest) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = argt
            fn.restype = rest
        _lib = L
    return _lib


def check(ctx, rc):
    if rc != MGLC_OK:
        msg = lib().mglc_last_error(ctx).decode() if ctx else ""
        raise MglcError(rc, msg)
