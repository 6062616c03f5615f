"""The three bindings of the C-ABI agree on every parameter struct: the C
header (include/mglc.h), the ctypes structures (mglc_gb300/capi.py) and the
Fortran bind(C) types (fortran/mglc_iface.f90) list the same fields, in the
same order, with the same types, and ctypes computes the C sizes."""
import ctypes
import os
import re

import pytest

from mglc_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_TYPES = {"int": ctypes.c_int, "double": ctypes.c_double, "long long": ctypes.c_longlong,
           "float": ctypes.c_float}
PY_NAMES = {"mglc_lid_params": "LidParams", "mglc_thermal_params": "ThermalParams",
            "mglc_particle_params": "ParticleParams", "mglc_info": "Info",
            "mglc_particle2d_params": "Particle2DParams", "mglc_shear2d_params": "Shear2DParams",
            "mglc_lid2d_params": "Lid2DParams", "mglc_nure_status": "NuReStatus",
            "mglc_server_params": "ServerParams", "mglc_request": "Request",
            "mglc_request_result": "RequestResult", "mglc_server_stats": "ServerStats"}
F_KINDS = {"integer(c_int)": "int", "real(c_double)": "double", "integer(c_long_long)": "long long",
           "real(c_float)": "float"}


def c_structs():
    src = open(os.path.join(ROOT, "include", "mglc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (\w+) \{(.*?)\}\s*\1;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"^(long long|int|double|float)\s+(.*)$", decl)
            assert m, (name, decl)
            for item in m.group(2).split(","):
                item = item.strip()
                a = re.match(r"^(\w+)(?:\[(\d+)\])?$", item)
                assert a, (name, item)
                fields.append((a.group(1), m.group(1), int(a.group(2) or 1)))
        out[name] = fields
    return out


def f_types():
    src = open(os.path.join(ROOT, "fortran", "mglc_iface.f90")).read()
    out = {}
    for name, body in re.findall(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", src, flags=re.S):
        fields = []
        for line in body.splitlines():
            line = line.split("!!")[0].strip()
            if not line:
                continue
            kind, rest = [x.strip() for x in line.split("::")]
            for item in re.split(r",(?![^()]*\))", rest):
                item = item.split("=")[0].strip()
                a = re.match(r"^(\w+)(?:\((\d+)\))?$", item)
                assert a, (name, item)
                fields.append((a.group(1), F_KINDS[kind], int(a.group(2) or 1)))
        out[name] = fields
    return out


def test_header_structs_have_ctypes_twins():
    structs = c_structs()
    assert set(PY_NAMES) <= set(structs)
    for cname, pyname in PY_NAMES.items():
        cls = getattr(capi, pyname)
        want = []
        for fname, ctype, count in structs[cname]:
            t = C_TYPES[ctype]
            want.append((fname, t * count if count > 1 else t))
        got = list(cls._fields_)
        assert [f for f, _ in got] == [f for f, _ in want], cname
        for (f, a), (_, b) in zip(got, want):
            assert ctypes.sizeof(a) == ctypes.sizeof(b) and getattr(a, "_type_", a) == getattr(
                b, "_type_", b), (cname, f)


@pytest.mark.parametrize("name", ["mglc_lid_params", "mglc_thermal_params", "mglc_particle_params",
                                  "mglc_particle2d_params", "mglc_shear2d_params",
                                  "mglc_lid2d_params", "mglc_nure_status"])
def test_fortran_types_match_the_header(name):
    c = c_structs()[name]
    f = f_types()[name]
    assert [(n.lower(), t, k) for n, t, k in c] == [(n.lower(), t, k) for n, t, k in f], name
