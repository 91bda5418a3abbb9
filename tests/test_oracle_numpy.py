"""The vectorised NumPy FP64 restatement (oracle/np_ref.py, the CPU-baseline
leg in madflow's array style) against the C++ oracle: the same |M|^2 to
rounding for g g > t t~ + 0, 1, 2 gluons, and per helicity for gg > tt~."""
import numpy as np
import pytest

from conftest import GC10, GC11, GC12, MT, WT


@pytest.mark.parametrize("k", [2, 3, 4])
def test_numpy_restatement_matches_oracle(oracle, k):
    import np_ref

    T = oracle.TTNG(k)
    x = np.random.default_rng(70 + k).uniform(size=(64, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    ref = T.smatrix(p, T.params(MT, WT, GC10, GC11, GC12))
    got = np_ref.TTNG(k, T.colour).smatrix(p, MT, WT, GC10, GC11, GC12)
    assert np.max(np.abs(got / ref - 1)) < 1e-13


def test_numpy_partials_match_oracle(oracle):
    import np_ref

    T = oracle.TTNG(3)
    x = np.random.default_rng(9).uniform(size=(4, 14))
    p, *_ = oracle.ramboflow(x, 5, 13000.0, [MT, MT, 0.0])
    prm = T.params(MT, WT, GC10, GC11, GC12)
    plan = np_ref.TTNG(3, T.colour)
    for h in T.helicities[::5]:
        A = plan.partials(p, h, MT, WT, GC10, GC11, GC12)
        for e in range(len(p)):
            ref = T.partials(p[e], h, prm)
            # a partial amplitude sums terms that cancel to ~1e-5 of their
            # size (gauge cancellations), so its rounding is ~1e-11 of it
            assert np.max(np.abs(A[:, e] - ref)) <= 1e-8 * max(np.abs(ref).max(), 1e-300)
