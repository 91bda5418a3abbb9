"""The process generator (colour matrix, helicities, diagram counts) and the
generated recursion, compiled as host code, against the oracle (CPU only)."""
import ctypes

import numpy as np
import pytest

from conftest import GC10, GC11, GC12, MT, WT
from madflow_gb300 import codegen


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_colour_matrix_exact_vs_numeric(oracle, k):
    num, den = codegen.colour_matrix(k)
    C = np.array(num, dtype=np.float64) / den
    np.testing.assert_allclose(C, oracle.colour_matrix(k), atol=1e-12 * np.abs(C).max())
    assert np.array_equal(C, C.T)


def test_colour_matrix_ggttx_matches_reference():
    # tests/mockup_debug_me.py:506-507: cf = [[16,-2],[-2,16]], denom = 3
    num, den = codegen.colour_matrix(2)
    assert den == 3 and num == [[16, -2], [-2, 16]]


def test_diagram_counts():
    for k, n in codegen.KNOWN_DIAGRAMS.items():
        assert codegen.diagram_count(k) == n


def test_helicities_match_reference_order(golden, oracle):
    np.testing.assert_array_equal(np.array(codegen.helicities(2)), golden["me_ggttx_helicities"])
    for k in (3, 4):
        np.testing.assert_array_equal(np.array(codegen.helicities(k)), oracle.TTNG(k).helicities)


def test_denominators():
    assert codegen.denominator(2) == 256
    assert codegen.denominator(4) == 512  # identical final-state gluons


def test_colour_matrix_bf16_tf32_exact():
    """The integer colour numerators are exact in TF32 (10-bit mantissa) for
    24 flows: no split precision is needed for the matrix itself."""
    num, _ = codegen.colour_matrix(4)
    vals = np.unique(np.abs(np.array(num)))
    assert np.all(vals < 2**11)


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_generated_recursion_vs_oracle(host_lib, oracle, k):
    """FP64 generated code within 1e-12 of the oracle; FP32 (mixed) within 5e-5; through the
    run-time stage loop and through the kernels' compile-time driver with paired items."""
    T = oracle.TTNG(k)
    prm = T.params(MT, WT, GC10, GC11, GC12)
    rng = np.random.default_rng(11 + k)
    x = rng.uniform(size=(16, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    coup = np.array([GC10.real, 0.0, 0.0, GC11.imag, 0.0, GC12.imag])
    me0 = T.smatrix(p, prm)
    for prec, tol in ((0, 1e-12), (1, 5e-5)):
        for fn in (host_lib.me_host_smatrix, host_lib.me_host_smatrix_compiled):
            out = np.zeros(len(p))
            pc = np.ascontiguousarray(p)
            fn(k, prec, _dp(pc), ctypes.c_int64(len(p)), _dp(coup), ctypes.c_double(MT), ctypes.c_double(WT),
               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            assert np.max(np.abs(out / me0 - 1)) < tol, (k, prec, fn.__name__)


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_generated_per_helicity_vs_oracle(host_lib, oracle, k):
    """Per-helicity values (Matrix_<proc>.matrix) in MadGraph's helicity order."""
    T = oracle.TTNG(k)
    prm = T.params(MT, WT, GC10, GC11, GC12)
    x = np.random.default_rng(70 + k).uniform(size=(1, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    _, ref = T.smatrix(p, prm, per_helicity=True)
    coup = np.array([GC10.real, 0.0, 0.0, GC11.imag, 0.0, GC12.imag])
    out = np.zeros(T.ncomb)
    host_lib.me_host_helicities(k, _dp(np.ascontiguousarray(p[0])), _dp(coup), ctypes.c_double(MT),
                                ctypes.c_double(WT), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    np.testing.assert_allclose(out, ref[:, 0], rtol=1e-11, atol=1e-14 * np.abs(ref).max())


def test_colour_tc_operand_layout():
    """The tensor-core B operand holds C^T in the canonical K-major layout
    (8-row x 16-byte core matrices, LBO 128 bytes, SBO NPERM/4 x 128 bytes),
    every element once, padding rows zero."""
    num, _ = codegen.colour_matrix(4)
    npad, flat = codegen.colour_tc_operand(4)
    n = len(num)
    assert npad == 32 and len(flat) == npad * n
    sbo, lbo = (n // 4) * 32, 32
    seen = set()
    for r in range(npad):
        for c in range(n):
            off = (r // 8) * sbo + (c // 4) * lbo + (r % 8) * 4 + (c % 4)
            assert off not in seen
            seen.add(off)
            assert flat[off] == (num[c][r] if r < n else 0.0)
    assert len(seen) == len(flat)


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_compile_time_driver_bitwise_equal(host_lib, oracle, k):
    """The kernels' compile-time stage driver (paired top-line items from four
    gluons on) does per item the arithmetic of the run-time stage loop, so
    both give bitwise the same |M|^2, in FP64 and in FP32."""
    x = np.random.default_rng(90 + k).uniform(size=(8, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    coup = np.array([GC10.real, 0.0, 0.0, GC11.imag, 0.0, GC12.imag])
    pc = np.ascontiguousarray(p)
    for prec in (0, 1):
        outs = []
        for fn in (host_lib.me_host_smatrix, host_lib.me_host_smatrix_compiled):
            out = np.zeros(len(p))
            fn(k, prec, _dp(pc), ctypes.c_int64(len(p)), _dp(coup), ctypes.c_double(MT), ctypes.c_double(WT),
               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            outs.append(out)
        assert np.array_equal(outs[0], outs[1]), (k, prec)
