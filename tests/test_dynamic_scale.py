"""madflow's default scale choice (scripts/madflow_exec.py:428-434): without
--fixed_scale, every event gets mu_F = mu_R = (sum of the outgoing
transverse masses) / 2, m_T^2 = p.p + p_T^2 (phasespace.py:406-415), the
densities at mu^2, alpha_s(mu^2) and the couplings of model.evaluate(alpha_s)
per event (:446).  The synthetic densities carry no alpha_s, so alpha_s(mu^2)
runs at one loop with five flavours from alpha_s(M_Z^2) = 0.118.

The integrand applies the per-event couplings as (alpha_s(mu^2) /
alpha_s(M_Z^2))^k on |M|^2 at alpha_s(M_Z^2).  test_coupling_power pins that
identity to the matrix elements evaluated with the per-event couplings
themselves (every tree diagram of these processes has k strong vertices);
the oracle's dynamic-scale integrand is checked against its fixed-scale one
and mu restated here; the GPU integrand against the oracle (FP64 1e-12)."""
import numpy as np
import pytest

from conftest import MT, WT, rel_err, scaled_err

MZ = 91.1876


def alphas_ratio(alpha_mz, q2):
    b0 = 23.0 / (12.0 * np.pi)
    return 1.0 / (1.0 + alpha_mz * b0 * np.log(q2 / (MZ * MZ)))


def scale2(plab):
    """(sum over the outgoing particles of m_T / 2)^2 for lab-frame momenta
    (N, n, 4), as madflow_exec.py:429-430 forms it."""
    q = plab[:, 2:, :]
    m2 = q[..., 0] ** 2 - q[..., 1] ** 2 - q[..., 2] ** 2 - q[..., 3] ** 2
    pt = np.sqrt(q[..., 1] ** 2 + q[..., 2] ** 2)
    return (np.sqrt(m2 + pt**2).sum(-1) / 2.0) ** 2


def _couplings(a):
    g = 2.0 * np.sqrt(np.pi * a)
    return -g, 1j * g, 1j * g * g


@pytest.mark.parametrize("k", [2, 3, 4])
def test_coupling_power(oracle, k):
    """|M|^2(g g > t t~ + (k-2) g) with GC_10, GC_11, GC_12 of alpha_s equals
    |M|^2 at 0.118 times (alpha_s / 0.118)^k."""
    x = np.random.default_rng(70 + k).uniform(size=(40, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    T = oracle.TTNG(k)
    me0 = T.smatrix(p, T.params(MT, WT, *_couplings(0.118)))
    for a in (0.09, 0.13, 0.2):
        me = T.smatrix(p, T.params(MT, WT, *_couplings(a)))
        assert rel_err(me, me0 * (a / 0.118) ** k) < 1e-13


def test_coupling_power_quark_channels(oracle):
    """q q~ > t t~ scales as alpha_s^2, the three processes of p p > t t~ j
    with a light-quark line as alpha_s^3."""
    x = np.random.default_rng(77).uniform(size=(40, 10))
    p4, *_ = oracle.ramboflow(x, 4, 13000.0, [MT, MT])
    x = np.random.default_rng(78).uniform(size=(40, 14))
    p5, *_ = oracle.ramboflow(x, 5, 13000.0, [MT, MT, 0.0])
    g0 = _couplings(0.118)
    m0 = oracle.smatrix_uux_ttx(p4, MT, WT, g0[1])
    chans = ("uux_ttxg", "ug_ttxu", "uxg_ttxux")
    q0 = [oracle.smatrix_qq3(ch, p5, MT, WT, g0[0], g0[1]) for ch in chans]
    for a in (0.1, 0.15):
        g = _couplings(a)
        assert rel_err(oracle.smatrix_uux_ttx(p4, MT, WT, g[1]), m0 * (a / 0.118) ** 2) < 1e-13
        for i, ch in enumerate(chans):
            assert rel_err(oracle.smatrix_qq3(ch, p5, MT, WT, g[0], g[1]), q0[i] * (a / 0.118) ** 3) < 1e-13


CASES = [(2, 0, (0.0, 0.0, 0.0)), (3, 0, (30.0, 4.0, 0.0)), (4, 0, (60.0, 2.5, 0.4)), (2, 1, (0.0, 0.0, 0.0)),
         (3, 1, (30.0, 4.0, 0.0))]


def _cfg(k, pp, cuts, dyn):
    return [1, k, 13000.0, MT, WT, 0.118, *cuts, 0, pp, dyn]


@pytest.mark.parametrize("k,pp,cuts", CASES)
def test_oracle_dynamic_scale(oracle, k, pp, cuts):
    """The oracle at the dynamical scale equals its fixed-scale integrand
    times (alpha_s(mu^2) / 0.118)^k, mu from the lab-frame momenta restated
    here (the synthetic densities do not depend on Q: their lookup at mu^2
    returns the values at mt^2 up to rounding)."""
    x = np.random.default_rng(80 + k + 10 * pp).uniform(size=(400, 4 * k + 2))
    T = oracle.TTNG(k)
    f_fix = oracle.integrand(_cfg(k, pp, cuts, 0), x, T)
    f_dyn = oracle.integrand(_cfg(k, pp, cuts, 1), x, T)
    p, _, x1, x2 = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    mu2 = scale2(oracle.boost_to_lab(p, x1, x2))
    assert np.all(mu2 >= MT * MT * (1 - 1e-12))  # two tops: mu >= mt
    np.testing.assert_array_equal(f_dyn == 0, f_fix == 0)
    nz = f_fix != 0
    assert nz.sum() > 50
    r = alphas_ratio(0.118, mu2) ** k
    # near x -> 1 the densities vanish and their bicubic sums cancel, so
    # compare on the scale of the largest value, and relatively above 1e-6 of it
    assert scaled_err(f_dyn, f_fix * r) < 1e-13
    big = np.abs(f_fix) > 1e-6 * np.abs(f_fix).max()
    assert rel_err(f_dyn[big], (f_fix * r)[big]) < 1e-11
    assert np.all(r[nz] < 1.0)  # mu above M_Z: a smaller coupling


@pytest.mark.gpu
@pytest.mark.parametrize("k,pp,cuts", CASES)
def test_integrand_dynamic_scale(cuda, oracle, k, pp, cuts):
    """FusedIntegrand(..., q2="dynamic") in FP64 against the oracle's
    dynamic-scale integrand: cut decisions exact, values to 1e-12 of the
    largest."""
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=cuts[0], etamax=cuts[1], drmin=cuts[2], q2="dynamic",
                           precision=0, initial_states="pp" if pp else "gg")
    x = np.random.default_rng(90 + k + 10 * pp).uniform(size=(300, integ.n_dim))
    f = integ(x).cpu().numpy()
    fo = oracle.integrand(_cfg(k, pp, cuts, 1), x, oracle.TTNG(k))
    np.testing.assert_array_equal(f == 0, fo == 0)
    assert (fo != 0).sum() > 30
    assert scaled_err(f, fo) < 1e-12
    big = np.abs(fo) > 1e-6 * np.abs(fo).max()
    assert rel_err(f[big], fo[big]) < 1e-9


@pytest.mark.gpu
def test_dynamic_scale_rejected_without_pdf(cuda):
    """The dynamical scale needs the hadronic integrand (kind 1): madflow
    itself has no alpha_s source without a PDF set."""
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    with pytest.raises(_lib.MadflowError):
        FusedIntegrand(2, kind=0, sqrts=1000.0, q2="dynamic", precision=0)(np.random.default_rng(1).uniform(size=(8, 8)))
