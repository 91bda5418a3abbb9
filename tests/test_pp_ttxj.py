"""p p > t t~ j at leading order: the light-quark channels q q~ > t t~ g,
q g > t t~ q and q~ g > t t~ q~ beside g g > t t~ g, as madflow's p p > t t~ j
run sums its processes over their initial states and mirror images
(scripts/madflow_exec.py:444-458, utilities.py:25-39).

No reference output exists for these processes (the reference's tests freeze
only g g > t t~), so the oracle's HELAS evaluation is pinned to an
evaluation of the textbook Feynman rules (tests/feynman_rules.py: Dirac
matrices, explicit spinors and polarisations, explicit SU(3) colour sums),
which is itself checked against the published g g > t t~ and q q~ > t t~
results (Combridge, Nucl. Phys. B151 (1979) 429) and against gauge
invariance.  The GPU is compared with the oracle: FP64 1e-12, mixed by
quantiles."""
import ctypes

import numpy as np
import pytest

import feynman_rules as FR
from conftest import GC10, GC11, GS, MT, WT, rel_err, scaled_err

CHANNELS = {"uux_ttxg": FR.me2_uux_ttxg, "ug_ttxu": FR.me2_ug_ttxu, "uxg_ttxux": FR.me2_uxg_ttxux}


def _momenta(oracle, n, seed, sqrts=13000.0):
    x = np.random.default_rng(seed).uniform(size=(n, 14))
    p, *_ = oracle.ramboflow(x, 5, sqrts, [MT, MT, 0.0])
    return p


def _conserving(p):
    """The incoming momenta rebuilt from the sum of the outgoing ones: the
    batch Newton rule of ramboflow leaves some events' energy off by up to
    1e-7 GeV, and the two evaluations take the propagator momenta from
    different legs."""
    q = p.copy()
    P = p[:, 2:].sum(1)
    E, Pz = P[:, 0], P[:, 3]
    z = np.zeros_like(E)
    q[:, 0] = np.stack([(E + Pz) / 2, z, z, (E + Pz) / 2], -1)
    q[:, 1] = np.stack([(E - Pz) / 2, z, z, -(E - Pz) / 2], -1)
    return q


def _two_to_two(oracle, n, seed):
    x = np.random.default_rng(seed).uniform(size=(n, 8))
    p3, _, _ = oracle.rambo(x, 2, 1000.0, [MT, MT])
    pa = np.array([500.0, 0, 0, 500.0])
    pb = np.array([500.0, 0, 0, -500.0])
    return np.concatenate([np.tile(pa, (n, 1, 1)), np.tile(pb, (n, 1, 1)), p3], axis=1)


def test_feynman_rules_reproduce_the_analytic_2to2(oracle):
    """The checker's conventions (spinors, polarisations, vertices, the sign of
    the three-gluon vertex against the colour factors) on the processes with
    a published closed form."""
    p = _two_to_two(oracle, 40, 1)
    s = 1000.0 ** 2
    dot = FR.mdot
    t1, t2 = 2 * dot(p[:, 0], p[:, 2]) / s, 2 * dot(p[:, 1], p[:, 2]) / s
    rho = 4 * MT * MT / s
    gg = GS ** 4 * (1 / (6 * t1 * t2) - 3.0 / 8) * (t1 ** 2 + t2 ** 2 + rho - rho ** 2 / (4 * t1 * t2))
    assert rel_err(FR.me2_gg_ttx(p, MT, GS), gg) < 1e-12
    t, u = dot(p[:, 0] - p[:, 2], p[:, 0] - p[:, 2]), dot(p[:, 0] - p[:, 3], p[:, 0] - p[:, 3])
    m2 = MT * MT
    qq = (4.0 / 9.0) * GS ** 4 * ((m2 - t) ** 2 + (m2 - u) ** 2 + 2.0 * m2 * s) / s ** 2
    assert rel_err(FR.me2_uux_ttx(p, MT, WT, GS), qq) < 1e-12


@pytest.mark.parametrize("channel", sorted(CHANNELS))
def test_feynman_rules_gauge_invariance(oracle, channel, monkeypatch):
    """Ward identity: the gluon's polarisation replaced by its momentum
    gives zero (zero top width)."""
    p = _momenta(oracle, 20, 3)
    ref = CHANNELS[channel](p, MT, 0.0, GS)
    monkeypatch.setattr(FR, "polarisations", lambda k: [k / k[..., :1], k / k[..., :1]])
    assert np.abs(CHANNELS[channel](p, MT, 0.0, GS) / ref).max() < 1e-12


@pytest.mark.parametrize("channel", sorted(CHANNELS))
def test_oracle_matches_feynman_rules(oracle, channel):
    """Median 1e-13; the largest differences (1e-10) sit at nearly collinear
    gluons, where the remaining rounding of momentum conservation (1e-11 GeV
    in the transverse momenta) is amplified."""
    p = _conserving(_momenta(oracle, 60, 4))
    ref = CHANNELS[channel](p, MT, WT, GS)
    got = oracle.smatrix_qq3(channel, p, MT, WT, GC10, GC11, f32q=False)
    r = np.abs(got / ref - 1)
    assert np.median(r) < 1e-13 and r.max() < 1e-9
    # madflow's float32 sqrt(1/2) in the gluon polarisation: 3.4e-8 of |M|^2
    f32 = oracle.smatrix_qq3(channel, p, MT, WT, GC10, GC11, f32q=True)
    assert 1e-8 < np.abs(f32 / got - 1).max() < 1e-7


def test_colour_matrix_in_the_sources(oracle):
    """The colour matrix of the five diagrams (oracle) and its eigenvector
    form (CUDA) against the brute-force colour sum."""
    cm = FR._colour_matrix(FR._colour_light_line())
    want = np.array([[8, -1, 7, -2, -9j], [-1, 8, -2, 7, 9j], [7, -2, 8, -1, -9j], [-2, 7, -1, 8, 9j],
                     [9j, -9j, 9j, -9j, 18]]) / 3.0
    np.testing.assert_allclose(cm, want, atol=1e-13)
    a = np.random.default_rng(7).normal(size=(5, 2)) @ np.array([1.0, 1j])
    s1, s2, s3 = a[0] + a[1] + a[2] + a[3], a[0] - a[1] + a[2] - a[3], a[0] + a[1] - a[2] - a[3]
    eig = abs(s1) ** 2 + 1.5 * abs(s2 + 2j * a[4]) ** 2 + abs(s3) ** 2 / 6
    assert abs(np.real(a @ cm @ a.conj()) - eig) < 1e-12 * eig


def test_oracle_pp_jet_integrand_adds_the_quark_channels(oracle):
    cfg = [1, 3, 13000.0, MT, WT, 0.118, 30.0, 4.0, 0.0, 0]
    x = np.random.default_rng(2).uniform(size=(400, 14))
    fgg = oracle.integrand(cfg, x, oracle.TTNG(3))
    fpp = oracle.integrand(cfg + [1], x, oracle.TTNG(3))
    assert np.all(fpp >= fgg) and np.all((fpp > fgg) == (fpp > 0))
    share = 1.0 - fgg.sum() / fpp.sum()
    assert 0.05 < share < 0.6


# ---- GPU -----------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("channel", sorted(CHANNELS))
def test_gpu_qq3_vs_oracle(cuda, oracle, channel):
    from madflow_gb300 import matrix

    cls = {"uux_ttxg": matrix.Matrix_1_uux_ttxg, "ug_ttxu": matrix.Matrix_1_ug_ttxu,
           "uxg_ttxux": matrix.Matrix_1_uxg_ttxux}[channel]
    p = _momenta(oracle, 4001, 5)
    ref = oracle.smatrix_qq3(channel, p, MT, WT, GC10, GC11)
    fp64 = cls(precision=0).smatrix(p, MT, WT, GC10, GC11).cpu().numpy()
    assert rel_err(fp64, ref) < 1e-12
    mixed = cls(precision=1).smatrix(p, MT, WT, GC10, GC11).cpu().numpy()
    r = np.abs(mixed / ref - 1)
    assert np.median(r) < 1e-6 and np.quantile(r, 0.99) < 2e-5 and r.max() < 1e-3


def _cfg(pp, cuts=(30.0, 4.0, 0.0)):
    return [1, 3, 13000.0, MT, WT, 0.118, *cuts, 0, 1 if pp else 0]


@pytest.mark.gpu
def test_gpu_pp_jet_integrand_vs_oracle(cuda, oracle):
    from madflow_gb300.vegas import FusedIntegrand

    x = np.random.default_rng(6).uniform(size=(3000, 14))
    fo = oracle.integrand(_cfg(True), x, oracle.TTNG(3))
    cuts = dict(ptmin=30.0, etamax=4.0)
    f = FusedIntegrand(3, kind=1, sqrts=13000.0, precision=0, initial_states="pp", **cuts)(x).cpu().numpy()
    assert scaled_err(f, fo) < 1e-12
    big = np.abs(fo) > 1e-6 * np.abs(fo).max()
    assert rel_err(f[big], fo[big]) < 1e-9
    fm = FusedIntegrand(3, kind=1, sqrts=13000.0, precision=1, initial_states="pp", **cuts)(x).cpu().numpy()
    assert abs(fm.sum() / fo.sum() - 1.0) < 1e-5
    # cut decisions of the mixed path (FP32) may differ at the cut edges
    assert np.count_nonzero((fm != 0) != (fo != 0)) <= 2


@pytest.mark.gpu
def test_gpu_pp_jet_fused_iteration_vs_oracle(cuda, oracle):
    """One fused VEGAS iteration of p p > t t~ j (FP64) against the oracle's
    replay on the same Philox uniforms: sums to 1e-10, bins exact."""
    import torch

    from madflow_gb300.vegas import FusedIntegrand

    N, nb = 12000, 50
    integ = FusedIntegrand(3, kind=1, sqrts=13000.0, precision=0, initial_states="pp", ptmin=30.0, etamax=4.0)
    ndim = integ.n_dim
    grid = torch.linspace(0, 1, nb + 1, dtype=torch.float64, device="cuda").repeat(ndim, 1).contiguous()
    it = torch.tensor([2], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    integ.iteration(grid, 4, 0, it, N, res)
    r = res.cpu().numpy()
    u = oracle.uniforms(4, 0, 2, 0, N, ndim)
    xs, jac, bins = oracle.vegas_sample(grid.cpu().numpy(), u)
    f = oracle.integrand(_cfg(True), xs, oracle.TTNG(3))
    sums, hist = oracle.vegas_accumulate(f * jac / N, bins, nb)
    assert rel_err(r[:2], sums) < 1e-10
    assert scaled_err(r[2:].reshape(ndim, nb), hist) < 1e-10


@pytest.mark.gpu
def test_gpu_qq3_argument_checks(cuda):
    import torch

    from madflow_gb300 import _lib

    lib = _lib.load()
    ps = torch.zeros((5, 4, 4), dtype=torch.float64, device="cuda")
    out = torch.empty(4, dtype=torch.float64, device="cuda")
    coup = torch.zeros(6, dtype=torch.float64, device="cuda")
    f = lib.mf_smatrix_qq_ttxj
    assert f(1, 3, ps.data_ptr(), 4, MT, WT, coup.data_ptr(), 0, out.data_ptr(), None) == _lib.MF_ERR_ARG
    assert f(2, 0, ps.data_ptr(), 4, MT, WT, coup.data_ptr(), 0, out.data_ptr(), None) == _lib.MF_ERR_ARG
    assert f(1, 0, ps.data_ptr(), 0, MT, WT, coup.data_ptr(), 0, out.data_ptr(), None) == _lib.MF_OK
    assert ctypes is not None
