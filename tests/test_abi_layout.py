"""The three bindings of the C-ABI agree: the C header (include/mglc.h), the
ctypes structures (mglc_gb300/capi.py) and the Fortran bind(C) types and
interfaces (fortran/mglc_iface.f90) list the same struct fields in the same
order with the same types, and every C function has a Fortran interface with
the same arguments, each passed by value or by reference as C passes it."""
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
                                  "mglc_lid2d_params", "mglc_nure_status", "mglc_info",
                                  "mglc_server_params", "mglc_request", "mglc_request_result",
                                  "mglc_server_stats"])
def test_fortran_types_match_the_header(name):
    c = c_structs()[name]
    f = f_types()[name]
    assert [(n.lower(), t, k) for n, t, k in c] == [(n.lower(), t, k) for n, t, k in f], name


def c_functions():
    """name -> (return type, [(type, name)]) of every function include/mglc.h declares."""
    src = open(os.path.join(ROOT, "include", "mglc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"typedef struct \w+ \{.*?\}\s*\w+;", "", src, flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\s*\b(mglc_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        params = []
        for a in " ".join(args.split()).split(","):
            a = a.strip()
            if not a or a == "void":
                continue
            m = re.match(r"^(.*?)(\w+)$", a)
            params.append((m.group(1).replace("const", "").replace(" ", ""), m.group(2)))
        out[name] = (" ".join(ret.split()).replace("const ", ""), params)
    return out


def f_functions():
    """name -> (kind of result or None, [(decl type, is value, name)])."""
    src = open(os.path.join(ROOT, "fortran", "mglc_iface.f90")).read()
    src = re.sub(r"&\s*\n\s*", " ", src)  # join continuation lines
    body = src[src.index("    interface"):src.index("    end interface")]
    out = {}
    for m in re.finditer(r"^[ \t]*(?:([^\n]+?)[ \t]+)?(function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*"
                         r"bind\(C, name=\"(\w+)\"\)(.*?)end (?:function|subroutine)",
                         body, flags=re.S | re.M):
        rtype, kind, fname, args, cname, decls = m.groups()
        assert fname == cname, (fname, cname)
        names = [a.strip().lower() for a in args.split(",") if a.strip()]
        info = {}
        for line in decls.splitlines():
            line = line.split("!!")[0].strip()
            if "::" not in line or line.startswith("import"):
                continue
            left, right = [x.strip() for x in line.split("::")]
            parts = [p.strip() for p in re.split(r",(?![^()]*\))", left)]
            for item in re.split(r",(?![^()]*\))", right):
                nm = item.split("(")[0].strip().lower()
                info[nm] = (parts[0].lower(), "value" in parts[1:], "(" in item)
        out[cname] = (rtype.lower() if kind == "function" else None,
                      [(info[n][0], info[n][1], info[n][2], n) for n in names])
    return out


SCALAR = {"int": "integer(c_int)", "longlong": "integer(c_long_long)", "double": "real(c_double)"}
POINTEE = {"double*": "real(c_double)", "int*": "integer(c_int)", "longlong*": "integer(c_long_long)",
           "char*": "character(kind=c_char)", "float*": "real(c_float)"}


def test_fortran_interfaces_match_every_c_function():
    cf, ff = c_functions(), f_functions()
    assert set(cf) == set(ff), sorted(set(cf) ^ set(ff))
    for name, (ret, params) in cf.items():
        fret, fparams = ff[name]
        want_ret = {"int": "integer(c_int)", "void": None, "char*": "type(c_ptr)"}[ret.replace(" ", "")]
        assert fret == want_ret, (name, ret, fret)
        assert len(params) == len(fparams), name
        for (ctype, cname), (ftype, byval, arr, fname) in zip(params, fparams):
            where = (name, cname, fname)
            if "*" not in ctype:  # a scalar passed by value
                assert byval and ftype == SCALAR[ctype], where
            elif ctype.endswith("**"):  # an output handle
                assert ftype == "type(c_ptr)" and not byval, where
            elif ftype == "type(c_ptr)":  # any pointer passed as an address
                assert byval, where
            else:  # a by-reference dummy of the pointee's type
                assert not byval, where
                if ctype in POINTEE:
                    assert ftype == POINTEE[ctype], where
                else:
                    assert ftype == "type(%s)" % ctype.rstrip("*"), where
