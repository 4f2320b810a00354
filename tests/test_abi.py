"""The C-ABI library builds, loads and exports every symbol include/padeops_gb300.h
declares (no GPU needed; no compute calls)."""
import ctypes
import subprocess

import pytest

from padeops_gb300 import _lib as L


def test_header_symbols_exported(native_lib):
    syms = L.exported_symbols()
    assert len(syms) >= 50
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        assert hasattr(native_lib, s)


def test_status_strings(native_lib):
    for code in (0, 2, 3, 7, 21, 324, 1001, 1002, 1003, 1004, 1005, 1006):
        assert L.strerror(code) != "unknown status"


def test_init_argument_errors_without_gpu(native_lib):
    """Argument checks run before any device call and return the reference's codes."""
    h = ctypes.c_void_p()
    assert native_lib.pade_cd06_init(ctypes.byref(h), 5, 0.1, 1, 0, 0) == L.PADE_EREF_PERIODIC_N
    assert native_lib.pade_cd06_init(ctypes.byref(h), 7, 0.1, 0, 0, 0) == L.PADE_EREF_NONPERIODIC_N
    assert native_lib.pade_cd10_init(ctypes.byref(h), 7, 0.1, 1, 0, 0) == L.PADE_EREF_NONPERIODIC_N
    assert native_lib.pade_cf90_init(ctypes.byref(h), 9, 1) == L.PADE_EREF_FILTER_N
    assert native_lib.pade_cd06stagg_init_periodic(ctypes.byref(h), 4, 0.1) == L.PADE_EREF_STAGG_N
    assert native_lib.pade_cd06_init(ctypes.byref(h), 16, -1.0, 1, 0, 0) == L.PADE_EINVAL
    assert native_lib.pade_destroy(None) == L.PADE_EINVAL
    assert h.value is None


def test_python_mirror_surface():
    import padeops_gb300 as P

    for cls, names in [(P.cd06, ["init", "dd1", "dd2", "dd3", "d2d1", "d2d2", "d2d3", "destroy", "GetSize"]),
                       (P.cd10, ["init", "dd1", "dd2", "dd3", "d2d1", "d2d2", "d2d3", "destroy", "GetSize"]),
                       (P.cf90, ["init", "filter1", "filter2", "filter3", "destroy"]),
                       (P.gaussian, ["init", "filter1", "filter2", "filter3", "destroy"]),
                       (P.cd06stagg, ["init", "ddz_E2C", "ddz_C2E", "ddz_C2C", "ddz_E2E", "d2dz2_C2C", "d2dz2_E2E",
                                      "InterpZ_E2C", "InterpZ_C2E", "destroy"])]:
        for n in names:
            assert callable(getattr(cls, n)), (cls, n)


def test_use_before_init_raises():
    import padeops_gb300 as P

    with pytest.raises(L.PadeError):
        P.cd10().handle
