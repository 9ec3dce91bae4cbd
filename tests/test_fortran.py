"""The Fortran interface (include/helios_cc.f90) against the C header it binds.

CPU: every function helios_cc.h declares has an interface of the same name in
the module, and the module's derived types carry the C structs' fields in
order. GPU (where a Fortran compiler exists): the module and a program that
solves dodecahexaene through it compile, link against the engine and give
the golden energy.
"""
import json
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "helios_cc.h")
MODULE = os.path.join(ROOT, "include", "helios_cc.f90")


def _c_functions():
    return set(re.findall(r"\b(hx_[a-z_0-9]+)\s*\(", open(HEADER).read()))


def _struct_fields(name):
    text = open(HEADER).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        for part in re.sub(r"\[.*?\]", "", decl).split(","):
            fields.append(re.findall(r"[A-Za-z_][A-Za-z_0-9]*", part)[-1])   # the declarator's name
    return fields


def _type_fields(name):
    text = open(MODULE).read()
    body = re.search(r"type, bind\(c\), public :: %s\n(.*?)end type" % name, text, re.S).group(1)
    fields = []
    for line in body.splitlines():
        if "::" in line:
            for part in line.split("::")[1].split(","):
                fields.append(re.sub(r"\(.*\)", "", part.strip()))
    return fields


def test_module_declares_every_c_function():
    text = open(MODULE).read()
    bound = set(re.findall(r"bind\(c, name='(hx_[a-z_0-9]+)'\)", text))
    assert bound == _c_functions()


def test_module_parameters_are_the_header_constants():
    want = {k: int(v) for k, v in re.findall(r"^#define (HX_[A-Z0-9_]+) \(?(-?\d+)\)?", open(HEADER).read(), re.M)}
    text = re.sub(r"&\s*\n\s*", " ", open(MODULE).read())
    got = {}
    for decl in re.findall(r"parameter, public :: (.*)", text):
        got.update({k: int(v) for k, v in re.findall(r"(HX_[A-Z0-9_]+) = (-?\d+)", decl)})
    assert want and got == want


@pytest.mark.parametrize("name", ["hx_ppp_model", "hx_cc_params"])
def test_module_types_match_the_c_structs(name):
    assert _type_fields(name) == _struct_fields(name)


def _fortran():
    for fc in ("gfortran", "gfortran-13", "flang-new", "flang"):
        if shutil.which(fc):
            return shutil.which(fc)
    return None


@pytest.mark.gpu
def test_fortran_program_solves_dodecahexaene(tmp_path):
    fc = _fortran()
    if fc is None:
        pytest.skip("no Fortran compiler on this machine")
    from helios_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "dodecahexaene")
    subprocess.run([fc, "-O1", "-J", str(tmp_path), MODULE, os.path.join(ROOT, "tests", "fortran", "dodecahexaene.f90"),
                    "-o", exe, "-L" + os.path.dirname(lib), "-lhelios_gb300", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    gold = next(c for c in json.load(open(os.path.join(ROOT, "tests", "golden", "golden.json")))["cases"]
                if c["kind"] == "dodecahexaene")
    assert int(out[0]) == 1
    assert abs(float(out[3]) - gold["eref"]) < 1e-9
    assert abs((float(out[2]) - float(out[3])) - gold["ecorr_1e10"]) < 1e-8
