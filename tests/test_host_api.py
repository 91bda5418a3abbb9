"""Host-side parts of the drop-in API that run without a GPU: the couplings
module (madflow parameters.py) against the golden vectors made by the
reference's own code, and the phase-space cut variables and cut functions of
PhaseSpaceGenerator (madflow phasespace.py:405-478) against a restatement of
the reference formulas."""
import collections

import numpy as np
import pytest
import torch

from conftest import MT, WT


def test_alphas_to_gs_golden(golden):
    from madflow_gb300.parameters import _alphas_to_gs

    gs = _alphas_to_gs(golden["param_alphas"]).numpy()
    np.testing.assert_allclose(gs, golden["param_gs"], rtol=1e-15, atol=0)


def _mockup_model():
    from madflow_gb300.parameters import Model

    # the couplings of madflow's frozen g g > t t~ module (tests/mockup_debug_me.py:21-26)
    const = collections.namedtuple("constants", ["mdl_MT", "mdl_WT"])(MT, WT)
    funcs = collections.namedtuple("functions", ["GC_10", "GC_11"])(lambda gs: -gs, lambda gs: 1j * gs)
    return Model(const, funcs)


def test_model_frozen_golden(golden):
    """Model.freeze_alpha_s(0.118) + evaluate() (parameters.py:44-98): the
    constants then GC_10, GC_11 at float32(0.118), as the reference's
    float_me([alpha_s]) gives them."""
    m = _mockup_model()
    assert not m.frozen
    m.freeze_alpha_s(0.118)
    assert m.frozen
    vals = m.evaluate()
    assert vals[0] == MT and vals[1] == WT
    np.testing.assert_allclose(np.asarray(vals[2]), golden["param_frozen_gc10"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(np.asarray(vals[3]), golden["param_frozen_gc11"], rtol=1e-15, atol=0)
    with pytest.raises(ValueError):
        m.freeze_alpha_s(0.2)  # already frozen
    m.unfreeze()
    assert not m.frozen


def test_model_per_event_alpha_s(golden):
    """Unfrozen: couplings per event from a vector of alpha_s."""
    m = _mockup_model()
    a = torch.tensor(golden["param_alphas"])
    vals = m.evaluate(a)
    gs = golden["param_gs"]
    np.testing.assert_allclose(np.asarray(vals[2]), -gs, rtol=1e-15, atol=0)
    np.testing.assert_allclose(np.asarray(vals[3]), 1j * gs, rtol=1e-15, atol=0)


def test_model_parameter_lookup():
    m = _mockup_model()
    assert m.parse_parameter("ZERO") == 0.0
    assert m.parse_parameter("mdl_MT") == MT
    assert m.parse_parameter("GC_10")(2.0) == -2.0
    assert m.get_masses() == [MT]
    with pytest.raises(AttributeError):
        m.parse_parameter("mdl_MZ")


def _momenta(n=2000, seed=3):
    rng = np.random.default_rng(seed)
    p3 = rng.normal(scale=200.0, size=(n, 3, 3))
    m = np.array([0.0, 173.0, 50.0])
    e = np.sqrt((p3 ** 2).sum(-1) + m ** 2)
    return np.concatenate([e[..., None], p3], -1)  # (n, 3 particles, 4)


def test_cut_variables_match_reference_formulas():
    """pt, mt2, mt (phasespace.py:405-420) and eta (the pseudorapidity the
    fused kernels cut on) of every particle."""
    from madflow_gb300.phasespace import PhaseSpaceGenerator as G

    p = _momenta()
    t = torch.tensor(p)
    pt = np.sqrt(p[..., 1] ** 2 + p[..., 2] ** 2)
    m2 = p[..., 0] ** 2 - (p[..., 1:] ** 2).sum(-1)
    pabs = np.sqrt((p[..., 1:] ** 2).sum(-1))
    eta = 0.5 * np.log((pabs + p[..., 3]) / (pabs - p[..., 3]))
    np.testing.assert_allclose(G.pt(t).numpy(), pt, rtol=1e-14)
    np.testing.assert_allclose(G.mt2(t).numpy(), m2 + pt ** 2, rtol=1e-12)
    np.testing.assert_allclose(G.mt(t).numpy(), np.sqrt(m2 + pt ** 2), rtol=1e-12)
    np.testing.assert_allclose(G.eta(t).numpy(), eta, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("variable,particle,lo,hi", [("mt", 1, 200.0, 400.0), ("mt2", 1, 4.0e4, None),
                                                     ("eta", 2, -1.5, 1.5), ("pt", 0, None, 150.0),
                                                     ("mt", None, 180.0, None)])
def test_register_cut_selection(variable, particle, lo, hi):
    """register_cut (phasespace.py:424-478): strict inequalities against the
    thresholds held through float32 (float_me), on one particle or on a
    (n, 4) array when no particle is given."""
    from madflow_gb300.phasespace import PhaseSpaceGenerator as G

    gen = G(5, 13000.0, masses=[0.0, 173.0, 50.0])
    gen.register_cut(variable, particle=particle, min_val=lo, max_val=hi)
    p = _momenta()
    ps = torch.tensor(p if particle is not None else p[:, 1, :])
    got = gen._cuts[0](ps).numpy()
    q = p[:, particle, :] if particle is not None else p[:, 1, :]
    v = getattr(G, variable)(torch.tensor(q)).numpy()
    ok = np.ones(len(q), dtype=bool)
    if lo is not None:
        ok &= v > float(np.float32(lo))
    if hi is not None:
        ok &= v < float(np.float32(hi))
    np.testing.assert_array_equal(got, ok)
    assert 0 < ok.sum() < len(ok)


def test_register_cut_rejects_bad_input():
    from madflow_gb300.phasespace import PhaseSpaceGenerator as G

    gen = G(5, 13000.0)
    with pytest.raises(ValueError):
        gen.register_cut("rapidity", particle=2, min_val=0.0)
    with pytest.raises(ValueError):
        gen.register_cut("pt", particle=5, min_val=10.0)
