"""Loader of the CUDA library and thin ctypes bindings of its C ABI.

There is no fallback: if the library is missing or cannot be loaded, every
call raises.  Device arrays are passed as raw pointers (``tensor.data_ptr()``).
"""
import ctypes
import os
import re

from . import build as _build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "madflow_gb300.h")

_lib = None

c_int, c_int64, c_uint32, c_uint64, c_double = ctypes.c_int, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double
c_void_p, c_char_p = ctypes.c_void_p, ctypes.c_char_p
c_dp = ctypes.c_void_p  # device pointers are passed as integers

MF_OK, MF_ERR_ARG, MF_ERR_CUDA, MF_ERR_UNSUPPORTED, MF_ERR_CAPACITY, MF_ERR_NONFINITE, MF_ERR_STATE = range(7)
MF_STAGES = 4
MF_TUNE_VARIANTS = 8
MF_PREC_FP64, MF_PREC_MIXED = 0, 1
MF_NEWTON_BATCH, MF_NEWTON_PER_EVENT = 0, 1
MF_INITIAL_GG, MF_INITIAL_PP = 0, 1


class MadflowError(RuntimeError):
    """A madflow_gb300 C-ABI call returned an error status."""

    def __init__(self, status, where):
        lib = load()
        msg = lib.mf_status_string(status).decode()
        if status == MF_ERR_CUDA:
            msg += ": " + lib.mf_last_cuda_error().decode()
        super().__init__(f"{where}: {msg} (status {status})")
        self.status = status


class DeviceError(RuntimeError):
    """A kernel of a madflow_gb300 handle reported an error on the device
    (a bounded wait on the tensor cores ran out; the affected events got NaN)."""


MF_MAX_CUTS = 8
CUT_VARIABLES = {"pt": 0, "mt": 1, "mt2": 2, "eta": 3}


class Cut(ctypes.Structure):
    _fields_ = [("variable", c_int), ("particle", c_int), ("has_min", c_int), ("has_max", c_int),
                ("min_val", c_double), ("max_val", c_double)]


class IntegrandConfig(ctypes.Structure):
    _fields_ = [
        ("kind", c_int),
        ("sqrts", c_double),
        ("mt", c_double),
        ("wt", c_double),
        ("alpha_s", c_double),
        ("ptmin", c_double),
        ("etamax", c_double),
        ("drmin", c_double),
        ("q2", c_double),
        ("newton_rule", c_int),
        ("initial_states", c_int),
        ("events_limit", c_int64),
        ("ptmin_all", c_double),
        ("ncuts", c_int),
        ("cuts", Cut * MF_MAX_CUTS),
    ]


_SIGS = {
    "mf_version": (c_char_p, []),
    "mf_status_string": (c_char_p, [c_int]),
    "mf_last_cuda_error": (c_char_p, []),
    "mf_process_create": (c_int, [c_int, c_int, ctypes.POINTER(c_void_p)]),
    "mf_process_destroy": (c_int, [c_void_p]),
    "mf_process_info": (c_int, [c_void_p] + [ctypes.POINTER(c_int)] * 4 + [ctypes.POINTER(c_double)]),
    "mf_process_helicities": (c_int, [c_void_p, ctypes.POINTER(c_double)]),
    "mf_process_colour_matrix": (c_int, [c_void_p, ctypes.POINTER(c_double)]),
    "mf_smatrix": (c_int, [c_void_p, c_dp, c_int64, c_double, c_double, c_dp, c_int64, c_dp, c_dp, c_void_p]),
    "mf_rambo": (c_int, [c_dp, c_int64, c_int, c_dp, c_int64, ctypes.POINTER(c_double), c_int, c_dp, c_dp, c_void_p]),
    "mf_ramboflow": (c_int, [c_dp, c_int64, c_int, c_double, ctypes.POINTER(c_double), c_int, c_dp, c_dp, c_dp, c_dp,
                             c_void_p]),
    "mf_boost_to_lab": (c_int, [c_dp, c_int64, c_int, c_dp, c_dp, c_void_p]),
    "mf_ixxxxx": (c_int, [c_dp, c_int64, c_double, c_double, c_double, c_dp, c_void_p]),
    "mf_oxxxxx": (c_int, [c_dp, c_int64, c_double, c_double, c_double, c_dp, c_void_p]),
    "mf_vxxxxx": (c_int, [c_dp, c_int64, c_double, c_double, c_double, c_dp, c_void_p]),
    "mf_sxxxxx": (c_int, [c_dp, c_int64, c_double, c_dp, c_void_p]),
    "mf_FFV1_0": (c_int, [c_dp, c_dp, c_dp, ctypes.POINTER(c_double), c_int64, c_dp, c_void_p]),
    "mf_FFV1_1": (c_int, [c_dp, c_dp, ctypes.POINTER(c_double), c_double, c_double, c_int64, c_dp, c_void_p]),
    "mf_FFV1_2": (c_int, [c_dp, c_dp, ctypes.POINTER(c_double), c_double, c_double, c_int64, c_dp, c_void_p]),
    "mf_VVV1P0_1": (c_int, [c_dp, c_dp, ctypes.POINTER(c_double), c_double, c_double, c_int64, c_dp, c_void_p]),
    "mf_integrand_ndim": (c_int, [c_void_p, ctypes.POINTER(IntegrandConfig), ctypes.POINTER(c_int)]),
    "mf_integrand": (c_int, [c_void_p, ctypes.POINTER(IntegrandConfig), c_dp, c_int64, c_dp, c_void_p]),
    "mf_integrand_rows": (c_int, [c_void_p, ctypes.POINTER(IntegrandConfig), c_dp, c_int64, c_dp, c_void_p]),
    "mf_vegas_iteration": (c_int, [c_void_p, ctypes.POINTER(IntegrandConfig), c_dp, c_int, c_uint64, c_uint32, c_dp,
                                   c_int64, c_dp, c_dp, c_dp, c_void_p]),
    "mf_smatrix_multi": (c_int, [ctypes.POINTER(c_void_p), c_int, ctypes.POINTER(c_void_p),
                                 ctypes.POINTER(c_int64), c_double, c_double, c_dp, ctypes.POINTER(c_void_p), c_void_p]),
    "mf_vegas_events": (c_int, [c_void_p, ctypes.POINTER(IntegrandConfig), c_dp, c_int, c_uint64, c_uint32, c_int,
                                c_int64, c_dp, c_dp, c_void_p]),
    "mf_unweight": (c_int, [c_dp, c_int64, c_double, c_uint64, c_uint32, c_void_p, c_void_p]),
    "mf_vegas_accumulate": (c_int, [c_dp, c_dp, c_dp, c_int64, c_int, c_int, c_double, c_dp, c_void_p]),
    "mf_process_set_timing": (c_int, [c_void_p, c_int]),
    "mf_process_error_flags": (c_int, [c_void_p, ctypes.POINTER(c_int), c_int]),
    "mf_process_nonfinite": (c_int, [c_void_p, ctypes.POINTER(c_int64), c_int]),
    "mf_process_set_wait_limit": (c_int, [c_void_p, c_int]),
    "mf_process_tuning": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                  ctypes.POINTER(ctypes.c_float)]),
    "mf_process_set_tuning": (c_int, [c_void_p, c_int, c_int]),
    "mf_process_stage_ms": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "mf_process_scratch_bytes": (c_int, [c_void_p, ctypes.POINTER(c_int64)]),
    "mf_vegas_accumulate_noalloc": (c_int, [c_dp, c_dp, c_dp, c_int64, c_int, c_int, c_double, c_dp, c_void_p]),
    "mf_vegas_refine": (c_int, [c_dp, c_dp, c_int, c_int, c_double, c_void_p]),
    "mf_vegas_sample": (c_int, [c_dp, c_int, c_int, c_dp, c_int64, c_dp, c_dp, c_dp, c_void_p]),
    "mf_philox_uniforms": (c_int, [c_uint64, c_uint32, c_uint32, c_uint64, c_int64, c_int, c_dp, c_void_p]),
    "mf_pdf_xfx": (c_int, [c_dp, c_int64, c_double, c_dp, c_void_p]),
    "mf_pdf_xfx_flavour": (c_int, [c_int, c_dp, c_int64, c_double, c_dp, c_void_p]),
    "mf_smatrix_qq_ttx": (c_int, [c_int, c_dp, c_int64, c_double, c_double, c_dp, c_int64, c_dp, c_void_p]),
    "mf_smatrix_qq_ttxj": (c_int, [c_int, c_int, c_dp, c_int64, c_double, c_double, c_dp, c_int64, c_dp, c_void_p]),
    "mf_pq_forward": (c_int, [c_dp, c_dp, c_int64, c_int, c_int, c_dp, c_dp, c_void_p]),
    "mf_pq_inverse": (c_int, [c_dp, c_dp, c_int64, c_int, c_int, c_dp, c_dp, c_void_p]),
    "mf_pq_backward": (c_int, [c_dp, c_dp, c_dp, c_dp, c_int64, c_int, c_int, c_dp, c_dp, c_void_p]),
    "mf_flow_layer_density": (c_int, [c_dp, c_dp, c_int64, c_int, c_dp, c_int, c_dp, c_int, c_int] + [c_dp] * 7
                              + [c_void_p]),
    "mf_flow_layer_sample": (c_int, [c_dp, c_dp, c_int64, c_int, c_dp, c_int, c_dp, c_int, c_int] + [c_dp] * 7
                             + [c_void_p]),
    "mf_flow_layer_grad_workspace": (c_int, [c_int, c_int, c_int, ctypes.POINTER(c_int64)]),
    "mf_flow_layer_grad": (c_int, [c_dp, c_dp, c_dp, c_int64, c_int, c_dp, c_int, c_dp, c_int, c_int] + [c_dp] * 13
                           + [c_dp, c_int64, c_void_p]),
    "mf_flow_inv_layer_tc": (c_int, [c_dp, c_int64, c_int, c_dp, c_int, c_dp, c_int, c_int, c_dp, c_dp, c_dp, c_dp,
                                     c_dp, c_dp, c_dp, c_dp, c_void_p]),
    "mf_flow_inv_layer_tc_bf16": (c_int, [c_dp, c_int64, c_int, c_dp, c_int, c_dp, c_int, c_int, c_dp, c_dp, c_dp,
                                          c_dp, c_dp, c_dp, c_dp, c_dp, c_void_p]),
}


def declared_symbols():
    """Function names declared in include/madflow_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mf_[a-zA-Z0-9_]+)\s*\(", text)))


def load(build_if_missing=True):
    """Load (building first when needed) the library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and _build.needs_build():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"madflow_gb300 CUDA library not found at {path}; run madflow_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
    _lib = lib
    return lib


def call(name, *args):
    """Call a C-ABI function and raise MadflowError on a non-zero status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != MF_OK:
        raise MadflowError(st, name)
    return st


def dbl_array(values):
    arr = (c_double * len(values))(*values)
    return arr
