"""The C-ABI library builds, loads without a GPU and exports every function
include/madflow_gb300.h declares (no compute calls here)."""
import ctypes

from madflow_gb300 import _lib, build


def test_library_exports_header_symbols():
    lib = _lib.load()
    declared = _lib.declared_symbols()
    assert len(declared) > 20
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.mf_version().startswith(b"madflow_gb300")


def test_status_strings_and_argument_errors():
    lib = _lib.load()
    assert lib.mf_status_string(0) == b"ok"
    assert lib.mf_status_string(_lib.MF_ERR_ARG) == b"invalid argument"
    # argument checks happen before any device work
    h = ctypes.c_void_p()
    assert lib.mf_process_create(7, 0, ctypes.byref(h)) == _lib.MF_ERR_UNSUPPORTED
    assert lib.mf_process_create(2, 9, ctypes.byref(h)) == _lib.MF_ERR_ARG
    assert lib.mf_process_create(4, 1, None) == _lib.MF_ERR_ARG


def test_process_info_without_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.mf_process_create(4, 1, ctypes.byref(h)) == 0
    vals = [ctypes.c_int() for _ in range(4)]
    den = ctypes.c_double()
    assert lib.mf_process_info(h, *[ctypes.byref(v) for v in vals], ctypes.byref(den)) == 0
    assert [v.value for v in vals] == [6, 64, 24, 123]
    assert den.value == 512.0
    assert lib.mf_process_destroy(h) == 0


def test_library_is_in_tree():
    import os

    assert os.path.commonpath([build.LIB_PATH, build.HERE]) == build.HERE
