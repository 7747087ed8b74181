"""The Fortran bind(C) module (include/adpres_gb300_bind.f90) against the C
header: every interface binds a declared entry point, and every bind(C)
derived type has the fields of the C struct in the same order and of the
same kinds (checked against the ctypes mirror of the header, which the GPU
tests exercise)."""
import ctypes
import os
import re

from adpres_gb300 import _lib
from conftest import ROOT

F90 = os.path.join(ROOT, "include", "adpres_gb300_bind.f90")
STRUCTS = {"adp_geom": _lib.AdpGeom, "adp_opts": _lib.AdpOpts, "adp_report": _lib.AdpReport,
           "adp_fb_tables": _lib.AdpFbTables, "adp_trans_opts": _lib.AdpTransOpts,
           "adp_trans_result": _lib.AdpTransResult}


def _fortran_types():
    text = open(F90).read()
    out = {}
    for name, body in re.findall(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", text, flags=re.S):
        fields = []
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, names = [x.strip() for x in line.split("::")]
            k = {"integer(c_int)": "int", "real(c_double)": "double", "type(c_ptr)": "ptr"}[kind]
            fields += [(n.strip(), k) for n in names.split(",")]
        out[name] = fields
    return out


def _ctypes_fields(cls):
    out = []
    for name, t in cls._fields_:
        if t is ctypes.c_int:
            k = "int"
        elif t is ctypes.c_double:
            k = "double"
        else:
            assert t is ctypes.c_void_p or issubclass(t, ctypes._Pointer), (name, t)
            k = "ptr"
        out.append((name.rstrip("_"), k))
    return out


def test_every_bound_function_is_declared():
    from test_capi_symbols import declared_functions
    declared = set(declared_functions())
    bound = set(re.findall(r'bind\(C, name="(adp_\w+)"\)', open(F90).read()))
    assert bound and bound <= declared, sorted(bound - declared)


def test_bind_c_types_match_the_header_structs():
    types = _fortran_types()
    assert set(STRUCTS) <= set(types), sorted(set(STRUCTS) - set(types))
    for name, cls in STRUCTS.items():
        assert types[name] == _ctypes_fields(cls), name
