"""Build of the CUDA library ``libmadflow_gb300.so`` (sm_103a) with nvcc.

The process headers are generated first (``codegen.write_generated``); the
translation units are compiled in parallel and linked into one shared library
with a plain C ABI (``include/madflow_gb300.h``).  Output goes to
``madflow_gb300/_build/``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libmadflow_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
SOURCES = ["mf_core.cu", "mf_proc_k2.cu", "mf_proc_k3.cu", "mf_proc_k4.cu", "mf_proc_k5.cu", "mf_proc_multi.cu", "mf_flow.cu", "mf_flow_tc.cu", "mf_flow_train.cu"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build madflow_gb300")
    return path


def _deps():
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".cu", ".cuh", ".h"))]
    out.append(os.path.join(HERE, "codegen.py"))
    out.append(os.path.join(os.path.dirname(HERE), "include", "madflow_gb300.h"))
    return out


def needs_build():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link the library; returns its path."""
    from . import codegen

    codegen.write_generated(os.path.join(CSRC, "generated"))
    if not force and not needs_build():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True, cwd=CSRC)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-4000:]}")
        if verbose:
            print(r.stderr)
        return obj

    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    # the largest translation units first
    srcs.sort(key=lambda s: -os.path.getsize(os.path.join(CSRC, s)) if "k4" not in s else -1e12)
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import time

    t = time.time()
    print(build(force=True), f"{time.time() - t:.1f}s")
