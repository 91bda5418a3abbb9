import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


HOST_SO = os.path.join(ROOT, "tests", "host", "_build", "libme_host.so")


@pytest.fixture(scope="session")
def host_lib():
    """The generated recursion and the product's stage functions compiled as
    host code (tests/host/me_host.cu)."""
    import ctypes
    import subprocess

    from madflow_gb300 import codegen

    src = os.path.join(ROOT, "tests", "host", "me_host.cu")
    gen = os.path.join(ROOT, "madflow_gb300", "csrc", "generated")
    codegen.write_generated(gen)
    csrc = os.path.join(ROOT, "madflow_gb300", "csrc")
    deps = [src] + [os.path.join(gen, f) for f in os.listdir(gen)] + [
        os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cuh", ".h"))]
    if not os.path.exists(HOST_SO) or any(os.path.getmtime(d) > os.path.getmtime(HOST_SO) for d in deps):
        os.makedirs(os.path.dirname(HOST_SO), exist_ok=True)
        subprocess.run(["nvcc", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-x", "cu", src, "-o", HOST_SO],
                       check=True, capture_output=True)
    return ctypes.CDLL(HOST_SO)


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import madflow_gb300._lib as L

    L.load()
    return torch


# SM parameters of the frozen gg -> tt~ module (tests/mockup_debug_me.py:21-26)
MT = 173.0
WT = 1.4915000200271606
GS = 1.2177157847767195
GC10, GC11, GC12 = -GS, 1j * GS, 1j * GS * GS


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def scaled_err(a, b):
    """max |a-b| / max |b|: for arrays with entries that are zero or nearly so."""
    a = np.asarray(a)
    b = np.asarray(b)
    m = np.nanmax(np.abs(b)) if b.size else 1.0
    return float(np.nanmax(np.abs(a - b)) / m) if a.size else 0.0
