"""p p > t t~ at leading order: the light-quark channel q q~ > t t~ beside
g g > t t~, as madflow's p p > t t~ run sums its processes over their
initial states and mirror images (scripts/madflow_exec.py:444-458,
utilities.py:25-39).

No reference output exists for q q~ > t t~ (the reference's tests freeze
only g g > t t~), so the oracle's evaluation (HELAS wavefunctions, the
fermion-pair current and FFV1_0, colour factor 2) is pinned to the published
analytic result (Combridge, Nucl. Phys. B151 (1979) 429):
  |M|^2 averaged = (4/9) g^4 [(m^2 - t)^2 + (m^2 - u)^2 + 2 m^2 s] / s^2,
and the GPU is compared with the oracle: FP64 1e-12, mixed 1e-5 relative.
The synthetic quark densities are checked against their defining sum rules."""
import ctypes
import math

import numpy as np
import pytest

from conftest import GC11, GS, MT, WT, rel_err, scaled_err


def _qq_momenta(oracle, n, sqrts, seed):
    x = np.random.default_rng(seed).uniform(size=(n, 8))
    p = oracle.rambo(x, 2, sqrts, [MT, MT])[0]
    e = sqrts / 2.0
    allp = np.zeros((n, 4, 4))
    allp[:, 0] = [e, 0.0, 0.0, e]
    allp[:, 1] = [e, 0.0, 0.0, -e]
    allp[:, 2:] = p
    return allp


def _combridge(allp):
    def dot(a, b):
        return a[..., 0] * b[..., 0] - (a[..., 1:] * b[..., 1:]).sum(-1)

    s = dot(allp[:, 0] + allp[:, 1], allp[:, 0] + allp[:, 1])
    t = dot(allp[:, 0] - allp[:, 2], allp[:, 0] - allp[:, 2])
    u = dot(allp[:, 0] - allp[:, 3], allp[:, 0] - allp[:, 3])
    m2 = MT * MT
    return (4.0 / 9.0) * GS ** 4 * ((m2 - t) ** 2 + (m2 - u) ** 2 + 2.0 * m2 * s) / s ** 2


@pytest.mark.parametrize("sqrts", [400.0, 1000.0, 13000.0])
def test_oracle_qq_ttx_matches_analytic(oracle, sqrts):
    allp = _qq_momenta(oracle, 3000, sqrts, 1)
    me = oracle.smatrix_uux_ttx(allp, MT, WT, GC11)
    assert rel_err(me, _combridge(allp)) < 1e-12


def test_synthetic_quark_densities(oracle):
    """Valence numbers 2 (u) and 1 (d), the sea momentum fractions, and the
    gluon unchanged by the flavour tables."""
    from scipy import integrate

    q2 = MT * MT

    def integ(f, weight):
        return integrate.quad(lambda x: oracle.pdf_xfx_flavour(f, np.array([x]), q2)[0] * weight(x), 1e-6, 1.0,
                              limit=500)[0]

    def valence(f):
        return integ(f, lambda x: 1.0 / x) - integ(-f, lambda x: 1.0 / x)

    # the tables start at x = 1e-6; below it the valence integrands
    # A x^-0.5 (1-x)^n hold A 2 sqrt(1e-6), with A = 2/B(1/2, 4), 1/B(1/2, 5)
    def beta(a, b):
        return math.exp(math.lgamma(a) + math.lgamma(b) - math.lgamma(a + b))

    tail = 2.0 * math.sqrt(1e-6)
    assert abs(valence(2) + 2.0 / beta(0.5, 4.0) * tail - 2.0) < 3e-4
    assert abs(valence(1) + 1.0 / beta(0.5, 5.0) * tail - 1.0) < 3e-4
    for f, frac in ((-2, 0.03), (-1, 0.03), (3, 0.015), (-3, 0.015), (4, 0.005), (-4, 0.005)):
        assert abs(integ(f, lambda x: 1.0) - frac) < 1e-4 * max(1.0, frac / 0.01)
    x = np.array([1e-4, 0.01, 0.3, 0.9])
    np.testing.assert_array_equal(oracle.pdf_xfx_flavour(21, x, q2), oracle.pdf_xfx(x, q2))


def test_oracle_pp_integrand_adds_the_quark_channel(oracle):
    """The p p integrand is the g g integrand plus w L_qq |M|^2(q q~)."""
    cfg = [1, 2, 13000.0, MT, WT, 0.118, 0.0, 0.0, 0.0, 0]
    x = np.random.default_rng(2).uniform(size=(400, 10))
    fgg = oracle.integrand(cfg, x, oracle.TTNG(2))
    fpp = oracle.integrand(cfg + [1], x, oracle.TTNG(2))
    assert np.all(fpp >= fgg) and np.any(fpp > fgg)


# ---- GPU -----------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("sqrts", [400.0, 13000.0])
def test_gpu_qq_ttx_vs_oracle(cuda, oracle, sqrts):
    from madflow_gb300.matrix import Matrix_1_uux_ttx

    allp = _qq_momenta(oracle, 5001, sqrts, 3)
    ref = oracle.smatrix_uux_ttx(allp, MT, WT, GC11)
    fp64 = Matrix_1_uux_ttx(precision=0).smatrix(allp, MT, WT, GC11).cpu().numpy()
    assert rel_err(fp64, ref) < 1e-12
    mixed = Matrix_1_uux_ttx(precision=1).smatrix(allp, MT, WT, GC11).cpu().numpy()
    assert rel_err(mixed, ref) < 1e-5


@pytest.mark.gpu
def test_gpu_quark_densities_vs_oracle(cuda, oracle):
    from madflow_gb300.utilities import synthetic_pdf

    x = np.exp(np.random.default_rng(4).uniform(np.log(1e-6), 0, size=500))
    for f in (21, 1, 2, 3, 4, -1, -2, -3, -4):
        g, go = synthetic_pdf(x, MT * MT, pdg=f).cpu().numpy(), oracle.pdf_xfx_flavour(f, x, MT * MT)
        assert scaled_err(g, go) < 1e-13, f
        big = go > 1e-6 * go.max()
        assert rel_err(g[big], go[big]) < 1e-10, f


def _cfg(pp, cuts=(0.0, 0.0, 0.0)):
    return [1, 2, 13000.0, MT, WT, 0.118, *cuts, 0, 1 if pp else 0]


@pytest.mark.gpu
def test_gpu_pp_integrand_vs_oracle(cuda, oracle):
    from madflow_gb300.vegas import FusedIntegrand

    x = np.random.default_rng(5).uniform(size=(2000, 10))
    fo = oracle.integrand(_cfg(True), x, oracle.TTNG(2))
    f = FusedIntegrand(2, kind=1, sqrts=13000.0, precision=0, initial_states="pp")(x).cpu().numpy()
    assert scaled_err(f, fo) < 1e-12
    big = np.abs(fo) > 1e-6 * np.abs(fo).max()
    assert rel_err(f[big], fo[big]) < 1e-9
    fm = FusedIntegrand(2, kind=1, sqrts=13000.0, precision=1, initial_states="pp")(x).cpu().numpy()
    assert abs(fm.sum() / fo.sum() - 1.0) < 1e-5
    # the quark channel's share of the integrand
    fgg = oracle.integrand(_cfg(False), x, oracle.TTNG(2))
    share = 1.0 - fgg.sum() / fo.sum()
    assert 0.01 < share < 0.5


@pytest.mark.gpu
def test_gpu_pp_fused_iteration_vs_oracle(cuda, oracle):
    """One fused VEGAS iteration of p p > t t~ against the oracle's VEGAS
    replay on the same Philox uniforms: bins exact, sums to 1e-10."""
    import torch

    from madflow_gb300.vegas import FusedIntegrand

    N, nb = 20000, 50
    integ = FusedIntegrand(2, kind=1, sqrts=13000.0, precision=0, initial_states="pp")
    ndim = integ.n_dim
    grid = torch.linspace(0, 1, nb + 1, dtype=torch.float64, device="cuda").repeat(ndim, 1).contiguous()
    it = torch.tensor([1], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    integ.iteration(grid, 4, 0, it, N, res)
    r = res.cpu().numpy()
    u = oracle.uniforms(4, 0, 1, 0, N, ndim)
    xs, jac, bins = oracle.vegas_sample(grid.cpu().numpy(), u)
    f = oracle.integrand(_cfg(True), xs, oracle.TTNG(2))
    sums, hist = oracle.vegas_accumulate(f * jac / N, bins, nb)
    assert rel_err(r[:2], sums) < 1e-10
    assert scaled_err(r[2:].reshape(ndim, nb), hist) < 1e-10


@pytest.mark.gpu
def test_gpu_pp_unsupported_combinations(cuda):
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    with pytest.raises(_lib.MadflowError):
        FusedIntegrand(4, kind=1, sqrts=13000.0, precision=0, initial_states="pp")(torch.rand((10, 18)))
    with pytest.raises(_lib.MadflowError):
        FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0, initial_states="pp")(torch.rand((10, 8)))
    # event output names one initial state per event: one channel only
    integ = FusedIntegrand(2, kind=1, sqrts=13000.0, precision=0, initial_states="pp")
    grid = torch.linspace(0, 1, 51, dtype=torch.float64, device="cuda").repeat(integ.n_dim, 1).contiguous()
    f = torch.empty(100, dtype=torch.float64, device="cuda")
    ps = torch.empty((100, 4, 4), dtype=torch.float64, device="cuda")
    st = _lib.load().mf_vegas_events(integ.matrix.handle, ctypes.byref(integ._cs), grid.data_ptr(), 50, 4, 0, 0, 100,
                                     f.data_ptr(), ps.data_ptr(), None)
    assert st == _lib.MF_ERR_UNSUPPORTED
