"""Independent physics checks of the tt~ + gluons matrix elements, all in the
oracle: the colour-ordered recursion reproduces madflow's frozen gg -> tt~
module, is gauge invariant (BRST: a gluon polarisation replaced by its
momentum gives zero), and agrees with a colour-dressed evaluation of the full
QCD Feynman rules for explicit colours."""
import itertools

import numpy as np
import pytest

from conftest import GC10, GC11, GC12, MT, WT, rel_err


def _point(oracle, k, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(size=(1, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    return p[0]


def test_recursion_reproduces_mockup(golden, oracle):
    T = oracle.TTNG(2)
    me = T.smatrix(golden["me_ggttx_p"], T.params(MT, WT, GC10, GC11, GC12))
    assert rel_err(me, golden["me_ggttx_smatrix"]) < 1e-12


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_gauge_invariance(oracle, k):
    T = oracle.TTNG(k)
    prm = T.params(MT, 0.0, GC10, GC11, GC12)  # zero width: exact gauge invariance
    p = _point(oracle, k, 5 + k)
    hels = T.helicities
    scale = max(np.abs(T.partials(p, h, prm)).max() for h in hels[:: max(1, len(hels) // 8)])
    for h in hels[:: max(1, len(hels) // 4)]:
        for part in [0, 1] + list(range(4, k + 2)):
            hb = h.copy()
            hb[part] = 4.0
            assert np.abs(T.partials(p, hb, prm)).max() / scale < 1e-9


@pytest.mark.parametrize("k", [3, 4])
def test_colour_dressed_equals_ordered(oracle, k):
    T = oracle.TTNG(k)
    prm = T.params(MT, WT, GC10, GC11, GC12)
    rng = np.random.default_rng(100 + k)
    p = _point(oracle, k, 21 + k)
    h = T.helicities[rng.integers(T.ncomb)]
    A = T.partials(p, h, prm)
    perms = list(itertools.permutations(range(k)))
    checked = 0
    while checked < 6:
        cols = [int(c) for c in rng.integers(0, 8, size=k)] + [int(c) for c in rng.integers(0, 3, size=2)]
        pred = sum(oracle.colour_string([cols[s] for s in sig], cols[k], cols[k + 1]) * A[i]
                   for i, sig in enumerate(perms))
        if abs(pred) < 1e-6 * np.abs(A).max():
            continue
        d = oracle.ttng_dressed(k, p, h, cols, prm, s3=1.0, kappa=1.0)
        assert abs(d - pred) / abs(pred) < 1e-10
        checked += 1


def test_colour_sum_ggttx_bruteforce(oracle):
    T = oracle.TTNG(2)
    prm = T.params(MT, WT, GC10, GC11, GC12)
    p = _point(oracle, 2, 3)
    h = T.helicities[6]
    A = T.partials(p, h, prm)
    tot = sum(abs(oracle.ttng_dressed(2, p, h, [a, b, i, j], prm)) ** 2
              for a in range(8) for b in range(8) for i in range(3) for j in range(3))
    assert abs(tot / np.real(A @ T.colour @ A.conj()) - 1) < 1e-12


def test_ggttx_analytic(oracle):
    """LO gg -> QQbar summed |M|^2 (Combridge, Nucl. Phys. B151 (1979) 429):
    sum|M|^2/256 = g^4 (1/(6 t1 t2) - 3/8)(t1^2 + t2^2 + rho - rho^2/(4 t1 t2)),
    t1,2 = 2 p1.p3/s, 2 p2.p3/s (massive), rho = 4 m^2/s; width-free."""
    rng = np.random.default_rng(4)
    x = rng.uniform(size=(50, 8))
    p3, w, _ = oracle.rambo(x, 2, 1000.0, [MT, MT])
    s = 1000.0**2
    pa = np.array([500.0, 0, 0, 500.0])
    pb = np.array([500.0, 0, 0, -500.0])
    allp = np.concatenate([np.tile(pa, (50, 1, 1)), np.tile(pb, (50, 1, 1)), p3], axis=1)
    me = oracle.smatrix_ggttx(allp, MT, 0.0, GC10, GC11, f32q=False)
    dot = lambda a, b: a[..., 0] * b[..., 0] - (a[..., 1:] * b[..., 1:]).sum(-1)
    t1 = 2 * dot(pa, p3[:, 0]) / s
    t2 = 2 * dot(pb, p3[:, 0]) / s
    rho = 4 * MT**2 / s
    g4 = GC11.imag**4
    ana = g4 * (1 / (6 * t1 * t2) - 3.0 / 8) * (t1**2 + t2**2 + rho - rho**2 / (4 * t1 * t2))
    np.testing.assert_allclose(me, ana, rtol=1e-12)
