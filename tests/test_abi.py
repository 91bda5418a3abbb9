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


def test_flow_layer_argument_checks():
    """mf_flow_inv_layer_tc rejects the shapes its kernel does not cover
    before touching the device; an empty batch is a no-op."""
    lib = _lib.load()
    f = lib.mf_flow_inv_layer_tc
    f.restype = ctypes.c_int
    null = [None] * 8

    def call(n, dim, na, nb, K):
        return f(None, ctypes.c_int64(n), dim, None, na, None, nb, K, *null, None)

    assert call(0, 18, 9, 9, 8) == 0
    assert call(10, 18, 9, 9, 5) == _lib.MF_ERR_ARG      # K not in {4, 8, 16}
    assert call(10, 18, 0, 9, 8) == _lib.MF_ERR_ARG      # no conditioning inputs
    assert call(10, 40, 20, 20, 8) == _lib.MF_ERR_ARG    # more than 16 per half
    assert call(10, 10, 9, 9, 8) == _lib.MF_ERR_ARG      # na + nb > dim
    assert call(10, 32, 16, 16, 16) == _lib.MF_ERR_ARG   # 7 dimensions in the first chunk, 9 x 33 > 256 after
    assert call(10, 18, 9, 9, 8) == _lib.MF_ERR_ARG      # null buffers


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


def test_integrand_config_layout_matches_header(tmp_path):
    """The ctypes mirror of mf_integrand_config has the C struct's size and
    field offsets (compiled from the header with the host C compiler)."""
    import shutil
    import subprocess
    from pathlib import Path

    import pytest

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in _lib.IntegrandConfig._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"madflow_gb300.h\"\nint main(void) {\n"
                   + "  printf(\"%zu\\n\", sizeof(mf_integrand_config));\n"
                   + "".join(f"  printf(\"%zu\\n\", offsetof(mf_integrand_config, {f}));\n" for f in fields)
                   + "  return 0;\n}\n")
    inc = Path(__file__).resolve().parents[1] / "include"
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got[0] == ctypes.sizeof(_lib.IntegrandConfig)
    assert got[1:] == [getattr(_lib.IntegrandConfig, f).offset for f in fields]


def test_config_struct_layout_matches_header(tmp_path):
    """The ctypes mirror of mf_integrand_config and mf_cut has the size and
    field offsets a C compiler gives the header's structs."""
    import shutil
    import subprocess

    import pytest

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in _lib.IntegrandConfig._fields_]
    src = tmp_path / "layout.c"
    body = "".join(f'  printf("%zu\\n", offsetof(mf_integrand_config, {f}));\n' for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "madflow_gb300.h"\nint main(void) {\n'
                   '  printf("%zu\\n%zu\\n", sizeof(mf_integrand_config), sizeof(mf_cut));\n' + body +
                   '  return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(__import__("pathlib").Path(_lib.HEADER).parent), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(_lib.IntegrandConfig), ctypes.sizeof(_lib.Cut)] + [
        getattr(_lib.IntegrandConfig, f).offset for f in fields]
    assert got == want
