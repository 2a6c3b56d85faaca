"""The ctypes mirrors of the C ABI's parameter structs match the headers.

A field order or type that differs between include/*.h and the Python
bindings (geopvi_gb300/_native.py, geopvi_gb300/fwi3d.py) or the oracles'
front ends would pass every value shifted; this parses the headers' struct
definitions and compares names, order and C types.  No GPU.
"""
import ctypes
import os
import re

import pytest

from geopvi_gb300 import _native, fwi3d
from oracle import oracle as O2
from oracle import oracle3d as O3

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
CTYPE = {"int": ctypes.c_int, "float": ctypes.c_float, "double": ctypes.c_double}


def header_struct(header, name):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", text, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), CTYPE[ctype]) for n in names.split(",")]
    return fields


@pytest.mark.parametrize("header,name,struct", [
    ("geopvi_fwi2d.h", "gb_fwi2d_params", _native.CParams),
    ("geopvi_fwi2d.h", "gb_fwi2d_params", O2.CParams),
    ("geopvi_fwi3d.h", "gb_fwi3d_params", fwi3d.CParams3),
    ("geopvi_fwi3d.h", "gb_fwi3d_params", O3.CParams3),
])
def test_params_struct_matches_header(header, name, struct):
    assert [(f, t) for f, t in struct._fields_] == header_struct(header, name)


def test_acquisition_struct_matches_header():
    fields = header_struct_pointer("geopvi_fwi3d.h", "gb_fwi3d_acq")
    assert [f for f, _ in fwi3d.CAcq3._fields_] == fields == [f for f, _ in O3.CAcq3._fields_]


def header_struct_pointer(header, name):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", text, flags=re.S).group(1)
    return [re.search(r"\*\s*(\w+)\s*$", d.strip()).group(1) for d in body.split(";") if d.strip()]


def test_instance_struct_matches_header():
    text = open(os.path.join(INCLUDE, "geopvi_fwi2d.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct gb_fwi2d_instance\s*\{(.*?)\}\s*gb_fwi2d_instance;", text, flags=re.S).group(1)
    names = [re.search(r"(\w+)\s*$", d.strip()).group(1) for d in body.split(";") if d.strip()]
    assert names == [f for f, _ in _native.CInstance._fields_]
    assert _native.CInstance._fields_[0][1] is _native.CParams
