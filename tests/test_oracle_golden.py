"""The CPU oracle against golden vectors produced by running madflow's own
phasespace.py, wavefunctions_flow.py and tests/mockup_debug_me.py
(tests/golden/make_golden.py).  Pins the oracle before it is trusted."""
import numpy as np
import pytest

from conftest import GC10, GC11, MT, WT, rel_err, scaled_err


def test_reference_constants(golden, oracle):
    # float_me(python float) goes through float32 in the reference
    assert golden["const_PI"] == oracle.PI_F32
    assert golden["const_SQH"] == oracle.SQH_F32
    assert golden["const_ACC"] == np.float64(np.float32(1e-10))


@pytest.mark.parametrize("n", range(2, 8))
def test_rambo_massless(golden, oracle, n):
    p, w, _ = oracle.rambo(golden[f"rambo0_n{n}_x"], n, 7e3)
    assert rel_err(p, golden[f"rambo0_n{n}_p"]) < 1e-13 or scaled_err(p, golden[f"rambo0_n{n}_p"]) < 1e-14
    assert rel_err(w, golden[f"rambo0_n{n}_w"]) < 1e-13


def test_rambo_massless_volume(oracle):
    """test_ps.py:37-67: the massless RAMBO weight is the analytic volume."""
    from math import factorial, pi

    rng = np.random.default_rng(0)
    for n in range(2, 8):
        x = rng.uniform(size=(5, 4 * n))
        _, w, _ = oracle.rambo(x, n, 7e3, f32q=False)
        vol = (7e3 ** (2 * n - 4) / 2.0) / factorial(n - 1) / factorial(n - 2) / (4 * pi) ** (2 * n - 3)
        np.testing.assert_allclose(w, vol, rtol=1e-6)


def test_rambo_variable_sqrts(golden, oracle):
    p, w, _ = oracle.rambo(golden["rambo0_var_x"], 5, golden["rambo0_var_sqrts"])
    assert scaled_err(p, golden["rambo0_var_p"]) < 1e-14
    assert rel_err(w, golden["rambo0_var_w"]) < 1e-13


@pytest.mark.parametrize("name", ["tt", "ttg", "ttgg", "ttggg", "zh", "single"])
def test_rambo_massive_batch_newton(golden, oracle, name):
    """Massive rescaling with the reference's batch-wide Newton stopping rule."""
    meta = golden[f"rambom_{name}_meta"]
    n, sq, m = int(meta[0]), meta[1], meta[2:]
    p, w, _ = oracle.rambo(golden[f"rambom_{name}_x"], n, sq, m)
    assert scaled_err(p, golden[f"rambom_{name}_p"]) < 1e-14
    assert rel_err(w, golden[f"rambom_{name}_w"]) < 1e-13


@pytest.mark.parametrize("name", ["gg_ttx", "gg_ttxg", "gg_ttxgg", "gg_ttxggg", "massless5"])
def test_ramboflow(golden, oracle, name):
    meta = golden[f"flow_{name}_meta"]
    npar, sq, m = int(meta[0]), meta[1], meta[2:]
    m = None if np.all(m == 0) else m
    p, w, x1, x2 = oracle.ramboflow(golden[f"flow_{name}_x"], npar, sq, m)
    assert scaled_err(p, golden[f"flow_{name}_p"]) < 1e-14
    assert rel_err(w, golden[f"flow_{name}_w"]) < 1e-13
    assert rel_err(x1, golden[f"flow_{name}_x1"]) < 1e-15
    assert rel_err(x2, golden[f"flow_{name}_x2"]) < 1e-15


def test_on_shell_masses(oracle):
    """test_ps.py:96-106: outgoing invariant masses equal the input masses."""
    rng = np.random.default_rng(1)
    x = rng.uniform(size=(100, 10))
    p, w, x1, x2 = oracle.ramboflow(x, 4, 7e3, [50.0, 125.0])
    m2 = p[..., 0] ** 2 - (p[..., 1:] ** 2).sum(-1)
    np.testing.assert_allclose(m2[:, 0:2], 0.0, atol=1e-6)
    np.testing.assert_allclose(m2[:, 2], 50.0**2, atol=1e-4, rtol=1e-4)
    np.testing.assert_allclose(m2[:, 3], 125.0**2, atol=1e-4, rtol=1e-4)


def test_boost_to_lab(golden, oracle):
    p, w, x1, x2 = oracle.ramboflow(golden["psgen_lab_x"], 4, 7e3, [50.0, 125.0])
    lab = oracle.boost_to_lab(p, x1, x2)
    assert scaled_err(lab, golden["psgen_lab_p"]) < 1e-13
    assert rel_err(w, golden["psgen_lab_w"]) < 1e-13


def test_pt_cut_selection(golden, oracle):
    """test_ps.py:70-93: pT window on particle 3 selects the same events."""
    x = golden["psgen_cut_x"]
    p, w, _, _ = oracle.ramboflow(x, 5, 7e3, None)
    pt = np.sqrt(p[:, 3, 1] ** 2 + p[:, 3, 2] ** 2)
    mask = (pt > 60.0) & (pt < 300.0)
    np.testing.assert_array_equal(np.nonzero(mask)[0], golden["psgen_cut_idx"].ravel())
    assert scaled_err(p[mask], golden["psgen_cut_p"]) < 1e-14


def _wf_cases():
    for mass in (0.0, 173.0):
        for nhel in (-1.0, 1.0):
            for ns in (-1.0, 1.0):
                yield mass, nhel, ns


@pytest.mark.parametrize("mass,nhel,nsf", list(_wf_cases()))
def test_fermion_wavefunctions(golden, oracle, mass, nhel, nsf):
    tag = f"m{int(mass)}_h{int(nhel)}_s{int(nsf)}"
    pw = golden["wf_p"]
    assert scaled_err(oracle.ixxxxx(pw, mass, nhel, nsf), golden[f"wf_ix_{tag}"]) < 1e-15
    assert scaled_err(oracle.oxxxxx(pw, mass, nhel, nsf), golden[f"wf_ox_{tag}"]) < 1e-15


def test_vector_wavefunctions(golden, oracle):
    pw = golden["wf_p"]
    for mass in (0.0, 91.0):
        hels = (-1.0, 1.0, 4.0) if mass == 0.0 else (-1.0, 0.0, 1.0, 4.0)
        for nhel in hels:
            for nsv in (-1.0, 1.0):
                tag = f"m{int(mass)}_h{int(nhel)}_s{int(nsv)}"
                assert scaled_err(oracle.vxxxxx(pw, mass, nhel, nsv), golden[f"wf_vx_{tag}"]) < 1e-15, tag


def test_aloha(golden, oracle):
    fin, fout, v1, v2 = golden["aloha_fin"], golden["aloha_fout"], golden["aloha_v1"], golden["aloha_v2"]
    assert scaled_err(oracle.FFV1_0(fin, fout, v1, GC11), golden["aloha_FFV1_0"]) < 1e-14
    assert scaled_err(oracle.FFV1_1(fout, v1, GC11, MT, WT), golden["aloha_FFV1_1"]) < 1e-14
    assert scaled_err(oracle.FFV1_2(fin, v1, GC11, MT, WT), golden["aloha_FFV1_2"]) < 1e-14
    out = oracle.VVV1P0_1(v1, v2, GC10, 0.0, 0.0)
    ref = golden["aloha_VVV1P0_1"]
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    assert scaled_err(np.nan_to_num(out), np.nan_to_num(ref)) < 1e-14


def test_smatrix_ggttx(golden, oracle):
    """The frozen gg -> tt~ module, summed and per helicity."""
    me, hel = oracle.smatrix_ggttx(golden["me_ggttx_p"], MT, WT, GC10, GC11, per_helicity=True)
    assert rel_err(me, golden["me_ggttx_smatrix"]) < 1e-13
    assert scaled_err(hel[:, :8], golden["me_ggttx_matrix_hel"]) < 1e-13
    me2 = oracle.smatrix_ggttx(golden["flow_gg_ttx_p"], MT, WT, GC10, GC11)
    assert rel_err(me2, golden["me_flow_ggttx_smatrix"]) < 1e-13


def test_alphas_couplings(golden):
    a = golden["param_alphas"]
    np.testing.assert_allclose(golden["param_gs"].real, 2 * np.sqrt(np.pi * a), rtol=1e-15)
    # freeze_alpha_s goes through float_me([alpha_s]) -> float32
    a32 = np.float64(np.float32(0.118))
    np.testing.assert_allclose(golden["param_frozen_gc10"].real, -2 * np.sqrt(np.pi * a32), rtol=1e-15)
