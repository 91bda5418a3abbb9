"""madflow's --pt_cut (scripts/madflow_exec.py:396-401): the phase space
registers p_T > cut for every outgoing particle, the tops included
(PhaseSpaceGenerator.register_cut, phasespace.py:417-422, 458-466: the
threshold through float_me, so float32; decided on the momenta before the
boost to the lab frame).  Events failing it give 0.  The oracle is checked
against that rule restated here in NumPy; the GPU integrand against the
oracle (FP64: cut decisions exact, values 1e-12)."""
import numpy as np
import pytest

from conftest import MT, WT, rel_err, scaled_err

# uniform points put most of the partonic energy in the TeV range, so the
# thresholds sit near the middle of each process's smallest-p_T distribution
CASES = [(2, 0, 1000.0, (0.0, 0.0, 0.0)), (2, 0, 3000.0, (0.0, 0.0, 0.0)), (3, 0, 600.0, (30.0, 4.0, 0.0)),
         (4, 0, 300.0, (60.0, 2.5, 0.4)), (2, 1, 2000.0, (0.0, 0.0, 0.0)), (3, 1, 800.0, (30.0, 4.0, 0.0))]


def _cfg(k, pp, cut, gcuts):
    return [1, k, 13000.0, MT, WT, 0.118, *gcuts, 0, pp, 0, cut]


@pytest.mark.parametrize("k,pp,cut,gcuts", CASES)
def test_oracle_pt_cut(oracle, k, pp, cut, gcuts):
    x = np.random.default_rng(100 + k + 10 * pp + int(cut)).uniform(size=(500, 4 * k + 2))
    T = oracle.TTNG(k)
    f0 = oracle.integrand(_cfg(k, pp, 0.0, gcuts), x, T)
    f1 = oracle.integrand(_cfg(k, pp, cut, gcuts), x, T)
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    pt = np.sqrt(p[:, 2:, 1] ** 2 + p[:, 2:, 2] ** 2)
    keep = np.all(pt > np.float32(cut), axis=1)
    assert 0 < keep.sum() < len(keep)  # the cut removes some events and keeps others
    np.testing.assert_array_equal(f1, np.where(keep, f0, 0.0))


@pytest.mark.gpu
@pytest.mark.parametrize("k,pp,cut,gcuts", CASES)
def test_integrand_pt_cut(cuda, oracle, k, pp, cut, gcuts):
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=gcuts[0], etamax=gcuts[1], drmin=gcuts[2], pt_cut=cut,
                           precision=0, initial_states="pp" if pp else "gg")
    x = np.random.default_rng(110 + k + 10 * pp + int(cut)).uniform(size=(400, integ.n_dim))
    f = integ(x).cpu().numpy()
    fo = oracle.integrand(_cfg(k, pp, cut, gcuts), x, oracle.TTNG(k))
    np.testing.assert_array_equal(f == 0, fo == 0)
    assert (fo != 0).sum() > 20
    assert scaled_err(f, fo) < 1e-12
    big = np.abs(fo) > 1e-6 * np.abs(fo).max()
    assert rel_err(f[big], fo[big]) < 1e-9


@pytest.mark.gpu
def test_pt_cut_needs_hadronic_kind(cuda):
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    with pytest.raises(_lib.MadflowError):
        FusedIntegrand(2, kind=0, sqrts=1000.0, pt_cut=30.0, precision=0)(np.random.default_rng(1).uniform(size=(8, 8)))


# PhaseSpaceGenerator.register_cut tables (phasespace.py:424-478): pt, mt,
# mt2 of a named particle with a lower and/or upper bound; eta as well
TABLES = [
    (2, 0, [("pt", 2, 1500.0, None)]),
    (2, 1, [("mt", 3, None, 2500.0), ("pt", 2, 500.0, None)]),
    (3, 0, [("mt2", 4, 100.0**2, None), ("eta", 2, -1.5, 1.5)]),
    (4, 0, [("pt", 4, 200.0, 2000.0), ("mt", 2, 400.0, None), ("eta", 5, None, 2.0)]),
]


def _restate(p, cuts):
    """The cuts of PhaseSpaceGenerator on (N, n, 4) momenta, in NumPy."""
    keep = np.ones(p.shape[0], dtype=bool)
    for variable, particle, lo, hi in cuts:
        q = p[:, particle, :]
        pt = np.sqrt(q[:, 1] ** 2 + q[:, 2] ** 2)
        if variable == "pt":
            v = pt
        elif variable in ("mt", "mt2"):
            m2 = q[:, 0] * q[:, 0] - ((q[:, 1] * q[:, 1] + q[:, 2] * q[:, 2]) + q[:, 3] * q[:, 3])
            v = m2 + pt * pt
            v = np.sqrt(v) if variable == "mt" else v
        else:
            pabs = np.sqrt((q[:, 1] ** 2 + q[:, 2] ** 2) + q[:, 3] ** 2)
            v = 0.5 * np.log((pabs + q[:, 3]) / (pabs - q[:, 3]))
        if lo is not None:
            keep &= v > np.float32(lo)
        if hi is not None:
            keep &= v < np.float32(hi)
    return keep


@pytest.mark.parametrize("k,pp,cuts", TABLES)
def test_oracle_cut_table(oracle, k, pp, cuts):
    x = np.random.default_rng(120 + k + 10 * pp).uniform(size=(600, 4 * k + 2))
    T = oracle.TTNG(k)
    base = [1, k, 13000.0, MT, WT, 0.118, 0.0, 0.0, 0.0, 0, pp, 0, 0.0]
    f0 = oracle.integrand(base, x, T)
    f1 = oracle.integrand(base + oracle.cut_vector(cuts), x, T)
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    keep = _restate(p, cuts)
    assert 0 < keep.sum() < len(keep)
    np.testing.assert_array_equal(f1, np.where(keep, f0, 0.0))


@pytest.mark.gpu
@pytest.mark.parametrize("k,pp,cuts", TABLES)
def test_integrand_cut_table(cuda, oracle, k, pp, cuts):
    """FusedIntegrand(cuts=...) against the oracle, and the same table taken
    from a PhaseSpaceGenerator with the cuts registered."""
    from madflow_gb300.phasespace import PhaseSpaceGenerator
    from madflow_gb300.vegas import FusedIntegrand

    psg = PhaseSpaceGenerator(k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    for variable, particle, lo, hi in cuts:
        psg.register_cut(variable, particle=particle, min_val=lo, max_val=hi)
    assert psg.cut_table() == cuts
    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, cuts=psg.cut_table(), precision=0,
                           initial_states="pp" if pp else "gg")
    x = np.random.default_rng(130 + k + 10 * pp).uniform(size=(400, integ.n_dim))
    f = integ(x).cpu().numpy()
    base = [1, k, 13000.0, MT, WT, 0.118, 0.0, 0.0, 0.0, 0, pp, 0, 0.0]
    fo = oracle.integrand(base + oracle.cut_vector(cuts), x, oracle.TTNG(k))
    np.testing.assert_array_equal(f == 0, fo == 0)
    assert (fo != 0).sum() > 20
    assert scaled_err(f, fo) < 1e-12


@pytest.mark.gpu
def test_cut_table_rejects_bad_entries(cuda):
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    x = np.random.default_rng(1).uniform(size=(8, 10))
    with pytest.raises(_lib.MadflowError):  # particle 4 of a four-particle process
        FusedIntegrand(2, kind=1, sqrts=13000.0, cuts=[("pt", 4, 10.0, None)], precision=0)(x)
    with pytest.raises(ValueError):
        FusedIntegrand(2, kind=1, sqrts=13000.0, cuts=[("ht", 2, 10.0, None)], precision=0)
    with pytest.raises(ValueError):
        FusedIntegrand(2, kind=1, sqrts=13000.0, cuts=[("pt", 2, 1.0, None)] * 9, precision=0)
