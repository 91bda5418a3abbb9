"""The per-event flop counts bench.py reports: the algorithmic count equals
the oracle's counting-scalar evaluation, the recycled count the product's
stage functions run with a counting scalar (in the form of the FP32 kernel)."""
import ctypes

import numpy as np
import pytest

import bench
from conftest import GC10, GC11, GC12, MT, WT


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_alg_flops(oracle, k):
    T = oracle.TTNG(k)
    x = np.random.default_rng(0).uniform(size=(1, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    assert T.flops(p[0], T.params(MT, WT, GC10, GC11, GC12)) == bench.ALG_FLOPS[k]


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_recycled_flops(host_lib, oracle, k):
    x = np.random.default_rng(1).uniform(size=(1, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    coup = np.array([GC10.real, 0.0, 0.0, GC11.imag, 0.0, GC12.imag])
    dp = ctypes.POINTER(ctypes.c_double)
    host_lib.me_host_flops.restype = ctypes.c_double
    n = host_lib.me_host_flops(k, np.ascontiguousarray(p[0]).ctypes.data_as(dp), coup.ctypes.data_as(dp),
                               ctypes.c_double(MT), ctypes.c_double(WT))
    assert n == bench.REC_FLOPS[k]
    assert n < bench.ALG_FLOPS[k]
