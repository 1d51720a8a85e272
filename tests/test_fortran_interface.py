"""Host-side interface consistency (no GPU): the ISO_C_BINDING Fortran module
and the Python ctypes mirror against the C header.

* every `bind(C, name=...)` entry of the Fortran module is declared in
  include/mflops_gb300.h;
* the Fortran `navier_params` type and the ctypes `NavierParams` list the
  fields of `mf_navier_params_t` in the header's order with matching types;
* the ctypes offsets and size agree with the C compiler's (gcc, when present).
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mflops_gb300.h")
FORTRAN = os.path.join(ROOT, "mflops3d-md_gb300", "fortran", "mflops_gpu_f.f90")


def header_text():
    with open(HEADER) as f:
        return f.read()


def c_struct_fields(name):
    text = re.sub(r"/\*.*?\*/", "", header_text(), flags=re.S)
    m = re.search(r"typedef struct \{(.*?)\}\s*" + name + r"\s*;", text, flags=re.S)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        ctype, names = re.match(r"((?:const )?\w+\s*\**)\s*(.*)", decl).groups()
        for nm in names.split(","):
            fields.append((nm.strip(), ctype.replace(" ", "")))
    return fields


def fortran_type_fields(name):
    with open(FORTRAN) as f:
        text = f.read()
    m = re.search(r"type, bind\(C\), public :: " + name + r"\n(.*?)end type " + name, text, flags=re.S)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        ftype, names = [p.strip() for p in line.split("::")]
        for nm in names.split(","):
            fields.append((nm.strip(), ftype.replace(" ", "")))
    return fields


C_TO_F = {"double": "real(c_double)", "int": "integer(c_int)", "constchar*": "type(c_ptr)"}
C_TO_CTYPES = {"double": ctypes.c_double, "int": ctypes.c_int, "constchar*": ctypes.c_char_p}


def test_fortran_entries_are_declared():
    with open(FORTRAN) as f:
        names = re.findall(r'bind\(C,\s*name="(\w+)"\)', f.read())
    assert names
    text = header_text()
    missing = [n for n in names if not re.search(r"\b" + n + r"\s*\(", text)]
    assert not missing, missing


def test_fortran_navier_params_match_header():
    c = c_struct_fields("mf_navier_params_t")
    f = fortran_type_fields("navier_params")
    assert [n for n, _ in f] == [n for n, _ in c]
    for (cn, ct), (_, ft) in zip(c, f):
        assert C_TO_F[ct] == ft, (cn, ct, ft)


def test_ctypes_navier_params_match_header(mf):
    c = c_struct_fields("mf_navier_params_t")
    py = mf.NavierParams._fields_
    assert [n for n, _ in py] == [n for n, _ in c]
    for (cn, ct), (_, pt) in zip(c, py):
        assert C_TO_CTYPES[ct] == pt, (cn, ct, pt)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_ctypes_navier_params_layout_matches_compiler(mf, tmp_path):
    fields = [n for n, _ in c_struct_fields("mf_navier_params_t")]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mflops_gb300.h"', "int main(void) {",
             '  printf("size %zu\\n", sizeof(mf_navier_params_t));']
    lines += ['  printf("%s %%zu\\n", offsetof(mf_navier_params_t, %s));' % (n, n) for n in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                 text=True).stdout.splitlines())
    assert int(out["size"]) == ctypes.sizeof(mf.NavierParams)
    for n in fields:
        assert int(out[n]) == getattr(mf.NavierParams, n).offset, n
