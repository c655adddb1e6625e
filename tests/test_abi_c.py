"""The ABI seen from C and Fortran (CPU only): a C program compiled against
include/pixelflow_gpu.h and linked to libpixelflow_gb300.so reports the
struct layout, which must equal the ctypes structs field by field; the
Fortran interface module's bind(C) types must list the header's fields in
the same order with matching kinds; and the C program's GPU-free calls into
the library (default options, the step-host plan, strerror) return what the
Python side sees."""
import ctypes
import json
import os
import re
import shutil
import subprocess

import pytest

from pixelflow_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pixelflow_gpu.h")
FORTRAN = os.path.join(ROOT, "pixelflow_gb300", "fortran", "pixelflow_gpu.f90")


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    out = tmp_path_factory.mktemp("abi") / "abi_layout"
    libdir = os.path.dirname(_lib.LIB_PATH)
    _lib.load()  # builds nothing; fails loudly if the library is missing
    subprocess.check_call(["gcc", "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "abi_layout.c"), "-o", str(out), "-L", libdir,
                           "-lpixelflow_gb300", "-Wl,-rpath," + libdir])
    return json.loads(subprocess.check_output([str(out)], text=True))


@pytest.mark.parametrize("cname,ctype", [("pf_params", _lib.PfParams), ("pf_options", _lib.PfOptions),
                                         ("pf_shape", _lib.PfShape), ("pf_batch_options", _lib.PfBatchOptions)])
def test_ctypes_layout_equals_c(c_layout, cname, ctype):
    fields = {k.split(".", 1)[1]: v for k, v in c_layout.items() if k.startswith(cname + ".")}
    assert [f for f, _ in ctype._fields_] == list(fields), cname
    for f, _ in ctype._fields_:
        desc = getattr(ctype, f)
        assert [desc.offset, desc.size] == fields[f], (cname, f)
    assert ctypes.sizeof(ctype) == c_layout[f"sizeof.{cname}"][1]


def test_c_caller_sees_library_defaults(c_layout):
    L = _lib.load()
    o = _lib.PfOptions()
    L.pf_default_options(ctypes.byref(o))
    assert c_layout["abi_version"][1] == L.pf_abi_version()
    assert c_layout["default.precision"][1] == o.precision == 0
    assert c_layout["default.use_graph"][1] == o.use_graph == 1
    assert c_layout["default.sor_path"][1] == o.sor_path == 0
    assert c_layout["batch.use_graph"][1] == 1 and c_layout["batch.cluster"][1] == 4
    assert c_layout["step_host_slabs_256"][1] > 1
    assert c_layout["strerror_timeout_len"][1] > 0


def _header_struct(name):
    text = open(HEADER).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, names = decl.split(None, 1)
        for nm in names.split(","):
            nm = nm.strip()
            m = re.match(r"(\w+)(\[(\d+)\])?", nm)
            out.append((m.group(1), typ, int(m.group(3) or 1)))
    return out


def _fortran_type(name):
    text = open(FORTRAN).read()
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type %s" % (name, name), text, re.S).group(1)
    out = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = line.split("::")
        for nm in names.split(","):
            nm = nm.strip()
            m = re.match(r"(\w+)(\((\d+)\))?", nm)
            out.append((m.group(1).lower(), kind.strip(), int(m.group(3) or 1)))
    return out


@pytest.mark.parametrize("name", ["pf_params", "pf_options"])
def test_fortran_bind_c_types_follow_the_header(name):
    kinds = {"int32_t": "integer(c_int32_t)", "double": "real(c_double)"}
    h = _header_struct(name)
    f = _fortran_type(name)
    assert [x[0].lower() for x in h] == [x[0] for x in f], name
    for (hn, ht, hc), (fn, fk, fc) in zip(h, f):
        assert kinds[ht] == fk and hc == fc, (name, hn, ht, fk)
