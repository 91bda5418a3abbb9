"""The per-event algorithmic flop counts bench.py reports equal the oracle's
counting-scalar evaluation."""
import numpy as np
import pytest

import bench
from conftest import GC10, GC11, GC12, MT, WT


@pytest.mark.parametrize("k", [2, 3, 4])
def test_alg_flops(oracle, k):
    T = oracle.TTNG(k)
    x = np.random.default_rng(0).uniform(size=(1, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    assert T.flops(p[0], T.params(MT, WT, GC10, GC11, GC12)) == bench.ALG_FLOPS[k]
