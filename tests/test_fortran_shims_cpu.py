"""The Fortran shim modules (fortran/*.F90) against the C ABI (no GPU, no Fortran compiler).

No Fortran compiler exists on either machine of this build, so the shims are checked
textually: every bind(C) name they declare is declared in include/padeops_gb300.h and
exported by the built library, every bind(C) interface passes as many arguments as the C
prototype takes, and every shim module keeps the reference's module name.
"""
import ctypes
import glob
import os
import re

import pytest

from padeops_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = {os.path.basename(p): open(p).read() for p in glob.glob(os.path.join(ROOT, "fortran", "*.F90"))}


def _c_prototypes():
    txt = re.sub(r"/\*.*?\*/", "", open(L.HEADER_PATH).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|const char\*)\s+(pade_\w+)\s*\(([^)]*)\)", txt):
        args = [a for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(1)] = len(args)
    return protos


def _f_interfaces():
    out = {}
    for name, src in SRC.items():
        for m in re.finditer(r"function\s+\w+\s*\(([^)]*)\)\s*(?:result\s*\(\w+\)\s*)?&?\s*(?:&\s*)?bind\(C,\s*name=\"(\w+)\"\)",
                             src.replace("&\n", " "), flags=re.I):
            args = [a for a in m.group(1).split(",") if a.strip()]
            out[m.group(2)] = (len(args), name)
    return out


def test_shim_modules_keep_the_reference_names():
    names = {re.search(r"^module\s+(\w+)", s, flags=re.M | re.I).group(1) for s in SRC.values()}
    for mod in ("cd06stuff", "cd10stuff", "cf90stuff", "gaussianstuff", "cd06staggstuff", "PadeDerOps",
                "spectralMod", "PadePoissonMod", "PoissonPeriodicMod"):
        assert mod in names, mod


def test_bind_c_interfaces_match_the_header_and_the_library():
    protos = _c_prototypes()
    ifaces = _f_interfaces()
    assert len(ifaces) >= 25
    lib_path = L.LIB_PATH
    lib = ctypes.CDLL(lib_path) if os.path.exists(lib_path) else None
    for cname, (nargs, where) in ifaces.items():
        assert cname in protos, (cname, where)
        assert protos[cname] == nargs, (cname, protos[cname], nargs)
        if lib is not None:
            assert hasattr(lib, cname), cname
