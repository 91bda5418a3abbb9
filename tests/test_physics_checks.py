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


def _lorentz(rng):
    """A random proper Lorentz transformation: rotation about a random axis,
    then a boost of speed < 0.8 along another random axis."""
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    th = rng.uniform(0, 2 * np.pi)
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
    n = rng.normal(size=3)
    n /= np.linalg.norm(n)
    b = rng.uniform(0.1, 0.8)
    g = 1 / np.sqrt(1 - b * b)
    L = np.eye(4)
    L[0, 0] = g
    L[0, 1:] = L[1:, 0] = g * b * n
    L[1:, 1:] = np.eye(3) + (g - 1) * np.outer(n, n)
    Rf = np.eye(4)
    Rf[1:, 1:] = R
    return L @ Rf


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_lorentz_invariance(oracle, host_lib, k):
    """|M|^2 summed over helicities is Lorentz invariant: the oracle and the
    product's generated evaluation (host harness, FP64) give the same value
    for boosted and rotated momenta.  Zero top width: a fixed width in the
    t-channel propagators breaks gauge invariance, and the sum over physical
    gluon polarisations then depends on the frame (at 2e-5 for some points).
    On-shell momenta: Newton iterated per event (the batch rule leaves the
    slowest events of a batch slightly off shell)."""
    import ctypes

    T = oracle.TTNG(k)
    prm = T.params(MT, 0.0, GC10, GC11, GC12)
    rng = np.random.default_rng(40 + k)
    x = rng.uniform(size=(64, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2), rule=oracle.NEWTON_PER_EVENT)
    q = np.einsum("ab,neb->nea", _lorentz(rng), p)
    for mom in (p, q):  # momentum conservation survives the transformation
        assert np.abs(mom[:, :2].sum(1) - mom[:, 2:].sum(1)).max() < 1e-9 * 13000.0
    me_p, me_q = T.smatrix(p, prm), T.smatrix(q, prm)
    assert rel_err(me_q, me_p) < 1e-10
    dp = ctypes.POINTER(ctypes.c_double)
    coup = np.array([GC10.real, 0.0, 0.0, GC11.imag, 0.0, GC12.imag])
    out = np.zeros(len(q))
    qc = np.ascontiguousarray(q)
    host_lib.me_host_smatrix(k, 0, qc.ctypes.data_as(dp), ctypes.c_int64(len(q)), coup.ctypes.data_as(dp),
                             ctypes.c_double(MT), ctypes.c_double(0.0), out.ctypes.data_as(dp))
    assert rel_err(out, me_p) < 1e-10
