"""Parity of the CUDA library with the reference (golden vectors from madflow's
own code) and with the CPU oracle, through the C ABI.  Tolerances: FP64 paths
1e-12 relative (per-event |M|^2) or tighter; VEGAS bin indices and Philox bits
exact; the mixed-precision |M|^2 path 1e-4 relative max."""
import numpy as np
import pytest

from conftest import GC10, GC11, GC12, MT, WT, rel_err, scaled_err

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def test_rambo_golden(cuda, golden):
    from madflow_gb300 import phasespace as ps

    for n in range(2, 8):
        p, w = ps.rambo(golden[f"rambo0_n{n}_x"], n, 7e3)
        assert scaled_err(_np(p), golden[f"rambo0_n{n}_p"]) < 1e-13
        assert rel_err(_np(w), golden[f"rambo0_n{n}_w"]) < 1e-13
    p, w = ps.rambo(golden["rambo0_var_x"], 5, cuda.tensor(golden["rambo0_var_sqrts"]))
    assert scaled_err(_np(p), golden["rambo0_var_p"]) < 1e-13
    for name in ["tt", "ttg", "ttgg", "ttggg", "zh", "single"]:
        meta = golden[f"rambom_{name}_meta"]
        n, sq, m = int(meta[0]), float(meta[1]), list(meta[2:])
        p, w = ps.rambo(golden[f"rambom_{name}_x"], n, sq, m)
        assert scaled_err(_np(p), golden[f"rambom_{name}_p"]) < 1e-13, name
        assert rel_err(_np(w), golden[f"rambom_{name}_w"]) < 1e-13, name


def test_ramboflow_golden(cuda, golden):
    from madflow_gb300 import phasespace as ps

    for name in ["gg_ttx", "gg_ttxg", "gg_ttxgg", "gg_ttxggg", "massless5"]:
        meta = golden[f"flow_{name}_meta"]
        npar, sq, m = int(meta[0]), float(meta[1]), list(meta[2:])
        m = None if not any(m) else m
        p, w, x1, x2 = ps.ramboflow(golden[f"flow_{name}_x"], npar, sq, m)
        assert scaled_err(_np(p), golden[f"flow_{name}_p"]) < 1e-13, name
        assert rel_err(_np(w), golden[f"flow_{name}_w"]) < 1e-13, name
        assert rel_err(_np(x1), golden[f"flow_{name}_x1"]) < 1e-15


def test_phase_space_generator_golden(cuda, golden):
    from madflow_gb300 import phasespace as ps

    gen = ps.PhaseSpaceGenerator(5, 7e3, algorithm="ramboflow")
    gen.register_cut("pt", particle=3, min_val=60, max_val=300.0)
    p, w, x1, x2, idx = gen(golden["psgen_cut_x"])
    np.testing.assert_array_equal(_np(idx).ravel(), golden["psgen_cut_idx"].ravel())
    assert scaled_err(_np(p), golden["psgen_cut_p"]) < 1e-13
    gen.clear_cuts()
    full = gen(golden["psgen_cut_x"])[0]
    assert full.shape[0] == golden["psgen_cut_x"].shape[0]
    gen2 = ps.PhaseSpaceGenerator(4, 7e3, masses=[50.0, 125.0], com_output=False)
    p, w, *_ = gen2(golden["psgen_lab_x"])
    assert scaled_err(_np(p), golden["psgen_lab_p"]) < 1e-13
    assert rel_err(_np(w), golden["psgen_lab_w"]) < 1e-13


def test_empty_batch(cuda):
    from madflow_gb300 import phasespace as ps
    from madflow_gb300.matrix import Matrix_1_gg_ttxgg

    p, w = ps.rambo(np.zeros((0, 8)), 2, 1000.0, [MT, MT])
    assert p.shape == (0, 2, 4) and w.shape == (0,)
    m = Matrix_1_gg_ttxgg()
    assert m.smatrix(np.zeros((0, 6, 4)), MT, WT, GC10, GC11, GC12).shape == (0,)


def test_wavefunctions_golden(cuda, golden):
    from madflow_gb300 import wavefunctions as wf

    pw = golden["wf_p"]
    for mass in (0.0, 173.0):
        for nhel in (-1.0, 1.0):
            for ns in (-1.0, 1.0):
                tag = f"m{int(mass)}_h{int(nhel)}_s{int(ns)}"
                assert scaled_err(_np(wf.ixxxxx(pw, mass, nhel, ns)), golden[f"wf_ix_{tag}"]) < 1e-15, tag
                assert scaled_err(_np(wf.oxxxxx(pw, mass, nhel, ns)), golden[f"wf_ox_{tag}"]) < 1e-15, tag
    for mass in (0.0, 91.0):
        for nhel in ((-1.0, 1.0, 4.0) if mass == 0.0 else (-1.0, 0.0, 1.0, 4.0)):
            for nsv in (-1.0, 1.0):
                tag = f"m{int(mass)}_h{int(nhel)}_s{int(nsv)}"
                assert scaled_err(_np(wf.vxxxxx(pw, mass, nhel, nsv)), golden[f"wf_vx_{tag}"]) < 1e-15, tag


def test_sxxxxx(cuda, golden):
    """sxxxxx (wavefunctions_flow.py:34-51) cannot run in the reference
    (tf.expand_dims on a rank-0 tensor), so there is no golden vector: the
    evident intent is the 3-slot scalar wavefunction [p0, p3] nss, [p1, p2]
    nss, 1."""
    from madflow_gb300 import wavefunctions as wf

    pw = golden["wf_p"]
    for nss in (-1.0, 1.0):
        out = _np(wf.sxxxxx(pw, nss))
        assert out.shape == (3, pw.shape[0])
        np.testing.assert_array_equal(out[0], (pw[:, 0] + 1j * pw[:, 3]) * nss)
        np.testing.assert_array_equal(out[1], (pw[:, 1] + 1j * pw[:, 2]) * nss)
        np.testing.assert_array_equal(out[2], np.ones(pw.shape[0], dtype=complex))


def test_aloha_golden(cuda, golden):
    from madflow_gb300 import aloha

    fin, fout, v1, v2 = golden["aloha_fin"], golden["aloha_fout"], golden["aloha_v1"], golden["aloha_v2"]
    assert scaled_err(_np(aloha.FFV1_0(fin, fout, v1, GC11)), golden["aloha_FFV1_0"]) < 1e-14
    assert scaled_err(_np(aloha.FFV1_1(fout, v1, GC11, MT, WT)), golden["aloha_FFV1_1"]) < 1e-14
    assert scaled_err(_np(aloha.FFV1_2(fin, v1, GC11, MT, WT)), golden["aloha_FFV1_2"]) < 1e-14
    out = _np(aloha.VVV1P0_1(v1, v2, GC10, 0.0, 0.0))
    ref = golden["aloha_VVV1P0_1"]
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    assert scaled_err(np.nan_to_num(out), np.nan_to_num(ref)) < 1e-14


def test_smatrix_ggttx_golden(cuda, golden):
    from madflow_gb300.matrix import Matrix_1_gg_ttx

    m = Matrix_1_gg_ttx(precision=0)
    me = _np(m.smatrix(golden["me_ggttx_p"], MT, WT, GC10, GC11))
    assert rel_err(me, golden["me_ggttx_smatrix"]) < 1e-12
    for i, h in enumerate(golden["me_ggttx_helicities"]):
        mh = _np(m.matrix(golden["me_ggttx_p"][:8], h, MT, WT, GC10, GC11))
        assert scaled_err(mh, golden["me_ggttx_matrix_hel"][i]) < 1e-12
    me2 = _np(m.smatrix(golden["flow_gg_ttx_p"], MT, WT, GC10, GC11))
    assert rel_err(me2, golden["me_flow_ggttx_smatrix"]) < 1e-12


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_smatrix_vs_oracle(cuda, oracle, k):
    from madflow_gb300.matrix import PROCESSES

    rng = np.random.default_rng(30 + k)
    N = 257  # not a multiple of the tile sizes
    x = rng.uniform(size=(N, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    T = oracle.TTNG(k)
    ref = T.smatrix(p, T.params(MT, WT, GC10, GC11, GC12))
    fp64 = _np(PROCESSES[k](precision=0).smatrix(p, MT, WT, GC10, GC11, GC12))
    assert rel_err(fp64, ref) < 1e-12
    mixed = _np(PROCESSES[k](precision=1).smatrix(p, MT, WT, GC10, GC11, GC12))
    assert rel_err(mixed, ref) < 1e-4


def test_smatrix_per_event_couplings(cuda, oracle):
    import torch

    from madflow_gb300.matrix import Matrix_1_gg_ttxg

    rng = np.random.default_rng(3)
    x = rng.uniform(size=(64, 14))
    p, *_ = oracle.ramboflow(x, 5, 13000.0, [MT, MT, 0.0])
    alphas = rng.uniform(0.1, 0.13, size=64)
    g = 2 * np.sqrt(np.pi * alphas)
    m = Matrix_1_gg_ttxg(precision=0)
    dev = torch.device("cuda")
    me = _np(m.smatrix(p, MT, WT, torch.tensor(-g + 0j, device=dev), torch.tensor(1j * g, device=dev),
                       torch.tensor(1j * g * g, device=dev)))
    T = oracle.TTNG(3)
    for e in (0, 17, 63):
        ref = T.smatrix(p[e:e + 1], T.params(MT, WT, -g[e], 1j * g[e], 1j * g[e] ** 2))[0]
        assert abs(me[e] / ref - 1) < 1e-12


def test_philox_bits_and_vegas_bins(cuda, oracle):
    import torch

    from madflow_gb300 import _lib

    N, ndim, nb = 1000, 18, 50
    u = torch.empty((ndim, N), dtype=torch.float64, device="cuda")
    _lib.call("mf_philox_uniforms", 4, 0, 3, 17, N, ndim, u.data_ptr(), None)
    torch.cuda.synchronize()
    uo = oracle.uniforms(4, 0, 3, 17, N, ndim)
    np.testing.assert_array_equal(_np(u).T, uo)
    rng = np.random.default_rng(0)
    grid = np.sort(np.concatenate([np.zeros((ndim, 1)), rng.uniform(size=(ndim, nb - 1)), np.ones((ndim, 1))], 1), 1)
    g = torch.tensor(grid, device="cuda")
    x = torch.empty_like(u)
    jac = torch.empty(N, dtype=torch.float64, device="cuda")
    bins = torch.empty((ndim, N), dtype=torch.int32, device="cuda")
    _lib.call("mf_vegas_sample", g.data_ptr(), ndim, nb, u.data_ptr(), N, x.data_ptr(), jac.data_ptr(),
              bins.data_ptr(), None)
    torch.cuda.synchronize()
    xo, jo, bo = oracle.vegas_sample(grid, uo)
    np.testing.assert_array_equal(_np(bins).T, bo)
    np.testing.assert_array_equal(_np(x).T, xo)
    assert rel_err(_np(jac), jo) < 1e-14


def test_vegas_refine_and_accumulate(cuda, oracle):
    import torch

    from madflow_gb300 import _lib

    rng = np.random.default_rng(1)
    ndim, nb, N = 6, 50, 5000
    grid = np.tile(np.linspace(0, 1, nb + 1), (ndim, 1))
    bins = rng.integers(0, nb, size=(N, ndim)).astype(np.int32)
    fw = rng.exponential(size=N)
    jac = np.ones(N)
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    fw_d = torch.tensor(fw, device="cuda")  # keep the device buffers alive across the launch
    jac_d = torch.tensor(jac, device="cuda")
    bins_d = torch.tensor(bins.T.copy(), device="cuda")
    _lib.call("mf_vegas_accumulate", fw_d.data_ptr(), jac_d.data_ptr(), bins_d.data_ptr(), N, ndim, nb, 1.0,
              res.data_ptr(), None)
    torch.cuda.synchronize()
    sums, hist = oracle.vegas_accumulate(fw, bins, nb)
    r = _np(res)
    assert rel_err(r[:2], sums) < 1e-12
    assert rel_err(r[2:].reshape(ndim, nb), hist) < 1e-12
    g = torch.tensor(grid, device="cuda")
    h = torch.tensor(hist, device="cuda")
    _lib.call("mf_vegas_refine", g.data_ptr(), h.data_ptr(), ndim, nb, 1.5, None)
    torch.cuda.synchronize()
    go = oracle.vegas_refine(grid, hist, 1.5)
    assert scaled_err(_np(g), go) < 1e-13
    assert np.all(np.diff(_np(g), axis=1) > 0)


def test_pdf(cuda, oracle):
    from madflow_gb300.utilities import synthetic_pdf

    x = np.exp(np.random.default_rng(2).uniform(np.log(1e-6), 0, size=500))
    g, go = _np(synthetic_pdf(x, MT * MT)), oracle.pdf_xfx(x, MT * MT)
    # log/exp differ by an ulp between CUDA and the host libm; near x -> 1 the
    # table values vanish and the bicubic sum cancels, so compare on the scale
    assert scaled_err(g, go) < 1e-13
    big = go > 1e-6 * go.max()
    assert rel_err(g[big], go[big]) < 1e-10


def _cfg_vec(kind, k, sqrts, ptmin=0.0, etamax=0.0, drmin=0.0):
    return [kind, k, sqrts, MT, WT, 0.118, ptmin, etamax, drmin, 0]


@pytest.mark.parametrize("k,cuts", [(3, (30.0, 4.0, 0.0)), (4, (60.0, 2.5, 0.4))])
def test_integrand_vs_oracle(cuda, oracle, k, cuts):
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=cuts[0], etamax=cuts[1], drmin=cuts[2], precision=0)
    rng = np.random.default_rng(40 + k)
    x = rng.uniform(size=(300, integ.n_dim))
    f = _np(integ(x))
    fo = oracle.integrand(_cfg_vec(1, k, 13000.0, *cuts), x, oracle.TTNG(k))
    np.testing.assert_array_equal(f == 0, fo == 0)
    nz = fo != 0
    assert nz.sum() > 10
    # |M|^2 agrees to 1e-12; the integrand also carries the PDF lookup (see test_pdf)
    assert scaled_err(f, fo) < 1e-12
    big = np.abs(fo) > 1e-6 * np.abs(fo).max()
    assert rel_err(f[big], fo[big]) < 1e-9


@pytest.mark.parametrize("k,cuts", [(3, (30.0, 4.0, 0.0)), (4, (60.0, 2.5, 0.4))])
def test_integrand_mixed_vs_oracle(cuda, oracle, k, cuts):
    """Mixed precision (FP32 phase space, cuts, PDF and wavefunctions; FP64
    rambo rescaling and propagator denominators) against the FP64 oracle:
    cut decisions may differ only for events within FP32 rounding of a cut
    boundary; elsewhere each value within 1e-4 of the largest and the sum
    within 1e-5."""
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=cuts[0], etamax=cuts[1], drmin=cuts[2], precision=1)
    rng = np.random.default_rng(50 + k)
    x = rng.uniform(size=(4000, integ.n_dim))
    f = _np(integ(x))
    fo = oracle.integrand(_cfg_vec(1, k, 13000.0, *cuts), x, oracle.TTNG(k))
    same = (f == 0) == (fo == 0)
    assert (~same).sum() <= 2
    assert (fo != 0).sum() > 100
    assert np.max(np.abs(f - fo)[same]) < 1e-4 * np.abs(fo).max()
    assert abs(f[same].sum() - fo[same].sum()) < 1e-5 * np.abs(fo[same]).sum()


def test_integrand_ggttx_fixed_sqrts(cuda, oracle):
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
    x = np.random.default_rng(5).uniform(size=(1000, 8))
    assert rel_err(_np(integ(x)), oracle.integrand(_cfg_vec(0, 2, 1000.0), x)) < 1e-11


def _oracle_iteration(oracle, cfg, plan, grid, seed, it, N, ndim, nb):
    u = oracle.uniforms(seed, 0, it, 0, N, ndim)
    x, jac, bins = oracle.vegas_sample(grid, u)
    f = oracle.integrand(cfg, x, plan)
    sums, hist = oracle.vegas_accumulate(f * jac / N, bins, nb)
    return sums, hist


def test_fused_iteration_vs_oracle(cuda, oracle):
    import torch

    from madflow_gb300.vegas import FusedIntegrand

    k, N, nb = 3, 20000, 50
    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, precision=0)
    ndim = integ.n_dim
    grid = torch.linspace(0, 1, nb + 1, dtype=torch.float64, device="cuda").repeat(ndim, 1).contiguous()
    it = torch.tensor([2], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    integ.iteration(grid, 4, 0, it, N, res)
    r1 = _np(res).copy()
    integ.iteration(grid, 4, 0, it, N, res)
    np.testing.assert_array_equal(_np(res), r1)  # bit-reproducible
    sums, hist = _oracle_iteration(oracle, _cfg_vec(1, k, 13000.0, 30.0, 4.0), oracle.TTNG(k), _np(grid), 4, 2, N,
                                   ndim, nb)
    assert rel_err(r1[:2], sums) < 1e-10
    assert scaled_err(r1[2:].reshape(ndim, nb), hist) < 1e-10


def test_vegas_ggttx_integral_vs_oracle(cuda, oracle):
    """Config-1 integral (g g > t t~ at sqrt(s) = 1 TeV): GPU VEGAS and the
    oracle's VEGAS replay agree within the combined statistical error."""
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    N, n_iter = 20000, 3
    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
    v = VegasFlow(8, N, use_graph=False)
    v.compile(integ)
    res, err = v.run_integration(n_iter)
    # oracle replay of the same iterations (same uniforms, same grid updates)
    grid = np.tile(np.linspace(0, 1, 51), (8, 1))
    wsum = wres = 0.0
    for it in range(n_iter):
        sums, hist = _oracle_iteration(oracle, _cfg_vec(0, 2, 1000.0), None, grid, 4, it, N, 8, 50)
        var = (N * sums[1] - sums[0] ** 2) / (N - 1)
        wsum += 1 / var
        wres += sums[0] / var
        grid = oracle.vegas_refine(grid, hist, 1.5)
    ro, eo = wres / wsum, 1 / np.sqrt(wsum)
    assert abs(res - ro) < 1e-9 * abs(ro)  # same samples: agreement far inside the error
    assert abs(res - ro) < 3 * np.hypot(err, eo)
    assert err / res < 0.01


def test_cuda_graph_replay_matches(cuda):
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=1)
    a = VegasFlow(8, 30000, use_graph=False)
    a.compile(integ)
    ra = a.run_integration(4)
    b = VegasFlow(8, 30000, use_graph=True)
    b.compile(integ)
    rb = b.run_integration(4)
    assert ra == rb


def test_stage_timing(cuda):
    """Stage timing: nothing before an uncaptured timed call, then four
    non-negative stage times whose matrix-element share is positive; the
    integrand values are unchanged by the timing events."""
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(3, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, precision=1)
    x = torch.rand((20000, integ.n_dim), dtype=torch.float64, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(3))
    f0 = integ(x)
    with pytest.raises(_lib.MadflowError):
        integ.stage_ms()
    integ.set_timing(True)
    f1 = integ(x)
    torch.cuda.synchronize()
    ms = integ.stage_ms()
    integ.set_timing(False)
    assert set(ms) == {"seed", "phase_space", "matrix_element", "accumulate"}
    assert all(v >= 0.0 for v in ms.values()) and ms["matrix_element"] > 0.0
    assert torch.equal(f0, f1)


def test_colour_tensor_core_vs_simt(cuda, oracle):
    """g g > t t~ g g in FP32: the colour sum on the tensor cores (TF32 split,
    the total) against the FP32 SIMT colour sum of the same amplitudes (the
    per-helicity outputs) and against the FP64 oracle; no tensor-core wait
    ran out."""
    import ctypes

    from madflow_gb300 import _lib
    from madflow_gb300.matrix import PROCESSES

    rng = np.random.default_rng(77)
    x = rng.uniform(size=(4099, 18))
    p, *_ = oracle.ramboflow(x, 6, 13000.0, [MT, MT, 0.0, 0.0])
    m = PROCESSES[4](precision=1)
    tot, hel = m.smatrix_per_helicity(p, MT, WT, GC10, GC11, GC12)
    tot, hel = _np(tot), _np(hel)
    simt = hel.sum(axis=0) / 512.0
    assert rel_err(tot, simt) < 1e-5
    T = oracle.TTNG(4)
    ref = T.smatrix(p[:257], T.params(MT, WT, GC10, GC11, GC12))
    assert rel_err(tot[:257], ref) < 1e-4
    flags = ctypes.c_int(-1)
    _lib.call("mf_process_error_flags", m.handle, ctypes.byref(flags), 1)
    assert flags.value == 0


def test_autotuner(cuda):
    """The first large enough call times every launch variant and keeps the
    fastest; a fixed configuration is honoured and unsupported ones are
    refused; results do not depend on the configuration."""
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=1)
    assert not integ.tuning()["tuned"]
    x = torch.rand((300_000, integ.n_dim), dtype=torch.float64, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(9))
    f_auto = integ(x)
    t = integ.tuning()
    assert t["tuned"]
    ms = t["variant_ms"]
    assert len(ms) == 8 and all(v > 0 for v in ms)
    best = min(range(8), key=lambda i: ms[i])
    assert (t["colour"], t["waves"]) == (best // 4, 1 << (best % 4))
    for colour in (0, 1):
        integ.matrix.set_tuning(colour, 2)
        f = integ(x)
        assert torch.allclose(f, f_auto, rtol=2e-5, atol=0.0)
    fp64 = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
    with pytest.raises(_lib.MadflowError):
        fp64.matrix.set_tuning(1, 8)
    assert fp64.tuning()["variant_ms"][4:] == [0.0] * 4 or not fp64.tuning()["tuned"]


@pytest.mark.parametrize("prec", [0, 1])
def test_smatrix_multi_process_launch(cuda, oracle, prec):
    """g g > t t~, t t~ g and t t~ g g batches of uneven sizes in one
    persistent launch give the single-process results (FP64: to rounding,
    1e-13, and 1e-11 for g g > t t~, whose single-process launch evaluates
    its three diagrams in one thread per event (as the reference's module
    does) while the persistent launch runs the colour-ordered recursion;
    mixed: within 1e-5, the single-process g g > t t~ g g colour sum runs on
    the tensor cores)."""
    from madflow_gb300.matrix import PROCESSES, smatrix_multi

    rng = np.random.default_rng(90)
    batches, singles = [], []
    for k, n in ((2, 1001), (3, 517), (4, 333)):
        x = rng.uniform(size=(n, 4 * k + 2))
        p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
        batches.append((PROCESSES[k](precision=prec), p))
        singles.append(_np(PROCESSES[k](precision=prec).smatrix(p, MT, WT, GC10, GC11, GC12)))
    outs = [_np(o) for o in smatrix_multi(batches, MT, WT, GC10, GC11, GC12)]
    for k, o, s in zip((2, 3, 4), outs, singles):
        if prec == 0:
            assert rel_err(o, s) < (1e-11 if k == 2 else 1e-13)
        else:
            assert rel_err(o, s) < 1e-5


def test_colour_tensor_core_120_flows(cuda, oracle):
    """g g > t t~ g g g in FP32: the 120-flow colour sum on the tensor cores
    (two 128-row halves, K in chunks of 40 flows) against the SIMT row loop
    on the same amplitudes and against the FP64 oracle."""
    import ctypes

    from madflow_gb300 import _lib
    from madflow_gb300.matrix import PROCESSES

    rng = np.random.default_rng(55)
    x = rng.uniform(size=(300, 22))
    p, *_ = oracle.ramboflow(x, 7, 13000.0, [MT, MT, 0.0, 0.0, 0.0])
    m = PROCESSES[5](precision=1)
    m.set_tuning(0, 8)
    simt = _np(m.smatrix(p, MT, WT, GC10, GC11, GC12))
    m.set_tuning(1, 8)
    tc = _np(m.smatrix(p, MT, WT, GC10, GC11, GC12))
    assert rel_err(tc, simt) < 1e-5
    T = oracle.TTNG(5)
    ref = T.smatrix(p[:40], T.params(MT, WT, GC10, GC11, GC12))
    assert rel_err(tc[:40], ref) < 1e-4
    flags = ctypes.c_int(-1)
    _lib.call("mf_process_error_flags", m.handle, ctypes.byref(flags), 1)
    assert flags.value == 0


def test_edge_cases_of_the_newer_entry_points(cuda):
    """Empty batches give empty results; invalid arguments give status codes,
    not faults: unweighting of nothing, a multi-process launch with an empty
    batch and repeated handles, event output with a bad iteration index, a
    tuning outside the variants, the integrand of no points."""
    import ctypes

    import torch

    from madflow_gb300 import _lib, lhe
    from madflow_gb300.config import stream_ptr
    from madflow_gb300.matrix import PROCESSES, smatrix_multi
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    idx, rel = lhe.unweight(torch.empty(0, dtype=torch.float64, device="cuda"), 1.0)
    assert idx.numel() == 0 and rel.numel() == 0
    with pytest.raises(_lib.MadflowError):
        lhe.unweight(torch.ones(4, dtype=torch.float64, device="cuda"), 0.0)
    m3, m4 = PROCESSES[3](precision=1), PROCESSES[4](precision=1)
    rng = np.random.default_rng(2)
    x = rng.uniform(size=(50, 18))
    from madflow_gb300.phasespace import ramboflow

    p4, *_ = ramboflow(x, 6, 13000.0, [MT, MT, 0.0, 0.0])
    outs = smatrix_multi([(m3, np.zeros((0, 5, 4))), (m4, p4)], MT, WT, GC10, GC11, GC12)
    assert outs[0].numel() == 0 and outs[1].numel() == 50
    assert torch.allclose(outs[1], m4.smatrix(p4, MT, WT, GC10, GC11, GC12), rtol=2e-5)
    with pytest.raises(_lib.MadflowError):
        smatrix_multi([(m4, p4), (m4, p4)], MT, WT, GC10, GC11, GC12)
    with pytest.raises(_lib.MadflowError):
        m4.set_tuning(1, 3)
    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=1)
    assert integ(torch.empty((0, 8), dtype=torch.float64, device="cuda")).numel() == 0
    v = VegasFlow(8, 1000, use_graph=False)
    f = torch.empty(10, dtype=torch.float64, device="cuda")
    ps = torch.empty((10, 4, 4), dtype=torch.float64, device="cuda")
    st = _lib.load().mf_vegas_events(integ.matrix.handle, ctypes.byref(integ._cs), v.grid.data_ptr(), v.nbins, 1, 0,
                                     -1, 10, f.data_ptr(), ps.data_ptr(), stream_ptr())
    assert st == _lib.MF_ERR_ARG


def test_fused_iteration_ggttxgg_vs_oracle(cuda, oracle):
    """c3 (g g > t t~ g g, pT > 60, |eta| < 2.5, dR > 0.4) in FP64: one fused
    iteration on a non-uniform grid against the oracle's replay of the same
    Philox uniforms — sums to 1e-10, every per-bin sum to 1e-10 scaled."""
    import torch

    from madflow_gb300.vegas import FusedIntegrand

    k, N, nb = 4, 3000, 50
    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=0)
    ndim = integ.n_dim
    rng = np.random.default_rng(8)
    steps = rng.uniform(0.5, 1.5, size=(ndim, nb))
    g = np.concatenate([np.zeros((ndim, 1)), np.cumsum(steps, axis=1)], axis=1)
    g /= g[:, -1:]
    g[:, -1] = 1.0
    grid = torch.tensor(g, dtype=torch.float64, device="cuda").contiguous()
    it = torch.tensor([5], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    integ.iteration(grid, 9, 0, it, N, res)
    r = _np(res)
    sums, hist = _oracle_iteration(oracle, _cfg_vec(1, k, 13000.0, 60.0, 2.5, 0.4), oracle.TTNG(k), g, 9, 5, N, ndim,
                                   nb)
    assert rel_err(r[:2], sums) < 1e-10
    assert scaled_err(r[2:].reshape(ndim, nb), hist) < 1e-10


def test_integrand_ggttxggg_vs_oracle(cuda, oracle):
    """c5 (g g > t t~ g g g) integrand in FP64 against the oracle, cuts on."""
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(5, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, drmin=0.2, precision=0)
    x = np.random.default_rng(45).uniform(size=(120, integ.n_dim))
    f = _np(integ(x))
    fo = oracle.integrand(_cfg_vec(1, 5, 13000.0, 30.0, 4.0, 0.2), x, oracle.TTNG(5))
    np.testing.assert_array_equal(f == 0, fo == 0)
    assert (fo != 0).sum() > 10
    assert scaled_err(f, fo) < 1e-12


def test_full_size_iteration_properties(cuda):
    """The benchmark's size (10^7 points of c3, mixed precision): properties
    that do not depend on the size.  Every point falls in exactly one bin per
    dimension, so each dimension's per-bin sums of w^2 add up to the total
    sum of w^2; the estimate is finite and positive; a replay of the same
    iteration is bit-identical."""
    import torch

    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=1)
    ndim, nb, N = integ.n_dim, 50, 10_000_000
    grid = torch.linspace(0, 1, nb + 1, dtype=torch.float64, device="cuda").repeat(ndim, 1).contiguous()
    it = torch.tensor([0], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    integ.iteration(grid, 4, 0, it, N, res)
    r = _np(res).copy()
    assert np.isfinite(r).all() and r[0] > 0 and r[1] > 0
    per_dim = r[2:].reshape(ndim, nb).sum(axis=1)
    assert np.abs(per_dim / r[1] - 1).max() < 1e-12
    integ.iteration(grid, 4, 0, it, N, res)
    assert np.array_equal(_np(res), r)


def test_phase_space_full_size_conservation(cuda):
    """ramboflow on 10^6 points (FP64): three-momentum conservation and
    positive finite weights always; energy conservation and on-shell masses
    to rounding when Newton iterates every event to convergence.  With
    madflow's batch rule the loop stops when the first event converges
    (phasespace.py:90-103) and the energies come from the step before the
    last update (phasespace.py:77-92), so the slowest of 10^6 events keep
    relative energy residuals up to ~1e-4 and top masses off by up to
    ~0.01 GeV (a quirk of the reference, reproduced); the reference's own
    test asks 1e-4 GeV on the masses, which most events meet."""
    from madflow_gb300.phasespace import NEWTON_BATCH, NEWTON_PER_EVENT, ramboflow

    k, N = 4, 1_000_000
    x = np.random.default_rng(17).uniform(size=(N, 4 * k + 2))
    mass = np.array([0.0, 0.0, MT, MT, 0.0, 0.0])
    for rule in (NEWTON_BATCH, NEWTON_PER_EVENT):
        p, w, x1, x2 = ramboflow(x, k + 2, 13000.0, [MT, MT, 0.0, 0.0], newton_rule=rule)
        p, w = _np(p), _np(w)
        roots = p[:, :2, 0].sum(axis=1)
        d = np.abs(p[:, :2].sum(axis=1) - p[:, 2:].sum(axis=1)) / roots[:, None]
        m2 = p[..., 0] ** 2 - (p[..., 1:] ** 2).sum(-1)
        dm = np.abs(np.sqrt(np.abs(m2[:, 2:4])) - MT)
        assert d[:, 1:].max() < 1e-12, rule
        assert np.isfinite(w).all() and (w > 0).all()
        if rule == NEWTON_PER_EVENT:
            assert d[:, 0].max() < 1e-12
            assert np.abs(m2 - mass**2).max() / 13000.0**2 < 1e-12
            assert dm.max() < 1e-6
        else:
            assert d[:, 0].max() < 1e-3
            assert dm.max() < 0.05
            assert (dm > 1e-4).mean() < 0.05


@pytest.mark.parametrize("k", [3, 4])
def test_lorentz_invariance_gpu(cuda, oracle, k):
    """The product's |M|^2 (FP64 and mixed) of boosted and rotated momenta
    equals that of the original ones.  Summed over helicities it is Lorentz
    invariant when the amplitude is gauge invariant: zero top width (a fixed
    width in the t-channel propagators breaks gauge invariance, and the
    polarisation sum then depends on the frame, at 2e-5 for some points), on
    shell momenta (Newton iterated per event; the batch rule leaves the
    slowest events of a batch slightly off shell)."""
    from madflow_gb300.matrix import PROCESSES
    from test_physics_checks import _lorentz

    rng = np.random.default_rng(60 + k)
    x = rng.uniform(size=(512, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2), rule=oracle.NEWTON_PER_EVENT)
    q = np.ascontiguousarray(np.einsum("ab,neb->nea", _lorentz(rng), p))
    m = PROCESSES[k](precision=0)
    a = _np(m.smatrix(p, MT, 0.0, GC10, GC11, GC12))
    b = _np(m.smatrix(q, MT, 0.0, GC10, GC11, GC12))
    assert rel_err(b, a) < 1e-10
    # mixed precision: its rounding differs between the frames, with the
    # spread of its error against FP64 (median ~3e-7, rare points ~1e-3)
    m = PROCESSES[k](precision=1)
    a = _np(m.smatrix(p, MT, 0.0, GC10, GC11, GC12))
    b = _np(m.smatrix(q, MT, 0.0, GC10, GC11, GC12))
    r = np.abs(b / a - 1)
    assert np.median(r) < 1e-5 and r.max() < 1e-2
