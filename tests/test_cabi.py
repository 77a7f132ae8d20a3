"""The C-ABI library builds, loads and exports every symbol include/csadv.h declares (CPU only)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "csadv.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(csadv_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from csadv import _lib
    return _lib.lib()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("csadv_plan_create", "csadv_time_step", "csadv_update_winds", "csadv_advance", "csadv_mass",
                 "csadv_errors", "csadv_set_tracer", "csadv_get_tracer", "csadv_divergence"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol():
    from csadv import _lib
    assert set(declared_functions()) <= set(_lib._SIGS)


def test_status_strings_without_gpu(lib):
    from csadv import _lib
    assert lib.csadv_version().startswith(b"csadv")
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8, -9):
        assert _lib.status_string(code) != "unknown status"


def test_plan_create_rejects_bad_arguments_before_touching_the_gpu(lib):
    from csadv import _lib
    o = _lib.Options()
    o.recon, o.dp, o.opsplit, o.et, o.mt, o.mf, o.vf, o.precision = 3, 1, 1, 3, 1, 3, 1, 64
    h = ctypes.c_void_p()
    bad = _lib.Options.from_buffer_copy(o)
    bad.recon = 7
    assert lib.csadv_plan_create(16, 0.01, 1, ctypes.byref(bad), None, ctypes.byref(h)) == _lib.ERR_OPTION
    bad = _lib.Options.from_buffer_copy(o)
    bad.opsplit = 3  # SP-PL07 with MT-0
    assert lib.csadv_plan_create(16, 0.01, 1, ctypes.byref(bad), None, ctypes.byref(h)) == _lib.ERR_OPTION_PAIR
    assert lib.csadv_plan_create(4, 0.01, 1, ctypes.byref(o), None, ctypes.byref(h)) == _lib.ERR_ARG
    for dt in (0.0, float("nan"), -5.0):  # dt < 0 is a CFL target (at most 4)
        assert lib.csadv_plan_create(16, dt, 1, ctypes.byref(o), None, ctypes.byref(h)) == _lib.ERR_ARG
    assert lib.csadv_plan_create(16, 0.01, 0, ctypes.byref(o), None, ctypes.byref(h)) == _lib.ERR_ARG
    assert lib.csadv_plan_create(16, 0.01, 1, None, None, ctypes.byref(h)) == _lib.ERR_ARG
    assert not h.value


def test_advance_host_rejects_a_missing_plan_without_gpu(lib):
    from csadv import _lib
    arr = (ctypes.c_void_p * 1)(None)
    assert lib.csadv_advance_host(None, 1, None, 0, None, 0, None) == _lib.ERR_ARG
    assert lib.csadv_advance_host(None, 1, arr, 0, arr, 1, None) == _lib.ERR_ARG
