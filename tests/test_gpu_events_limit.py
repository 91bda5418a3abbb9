"""events_limit on the fused pipeline: a call runs in consecutive slices of at
most events_limit events, as vegasflow hands madflow's integrand one slice of
events_limit events per call (scripts/madflow_exec.py:474-487).

* The sliced VEGAS iteration against the oracle replaying the same slices
  (the batch Newton rule of the massive phase space runs per slice): bins
  exact, sums to 1e-10.
* With the per-event Newton rule nothing depends on the slicing: f, the
  uniforms and the event momenta are bit-identical to one slice.
* A limit of at least the call's size is one slice, bit for bit.
* The handle's scratch holds two slices (the pipeline's two buffer sets).
* VegasFlow(events_limit=...) slices its fused iterations, graph or not."""
import ctypes

import numpy as np
import pytest

from conftest import MT, WT, rel_err, scaled_err

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _grid(torch, ndim, nb, seed):
    """A non-uniform VEGAS grid (sorted random edges, 0 and 1 kept)."""
    rng = np.random.default_rng(seed)
    inner = np.sort(rng.uniform(size=(ndim, nb - 1)), axis=1)
    g = np.concatenate([np.zeros((ndim, 1)), inner, np.ones((ndim, 1))], axis=1)
    return torch.tensor(g, dtype=torch.float64, device="cuda").contiguous()


@pytest.mark.parametrize("limit", [5000, 7919])
def test_sliced_iteration_vs_oracle(cuda, oracle, limit):
    torch = cuda
    from madflow_gb300.vegas import FusedIntegrand

    k, N, nb = 3, 18000, 50
    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, precision=0)
    ndim = integ.n_dim
    grid = _grid(torch, ndim, nb, 1)
    it = torch.tensor([3], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
    integ.iteration(grid, 4, 0, it, N, res, events_limit=limit)
    r = _np(res).copy()
    u = oracle.uniforms(4, 0, 3, 0, N, ndim)
    xs, jac, bins = oracle.vegas_sample(_np(grid), u)
    cfg = [1, k, 13000.0, MT, WT, 0.118, 30.0, 4.0, 0.0, 0]
    plan = oracle.TTNG(k)
    f = np.concatenate([oracle.integrand(cfg, xs[s:s + limit], plan) for s in range(0, N, limit)])
    sums, hist = oracle.vegas_accumulate(f * jac / N, bins, nb)
    assert rel_err(r[:2], sums) < 1e-10
    assert scaled_err(r[2:].reshape(ndim, nb), hist) < 1e-10


@pytest.mark.parametrize("prec", [0, 1])
def test_limit_at_or_above_n_is_one_slice(cuda, prec):
    torch = cuda
    from madflow_gb300.vegas import FusedIntegrand

    N, nb = 30000, 50
    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=prec)
    ndim = integ.n_dim
    grid = _grid(torch, ndim, nb, 2)
    it = torch.tensor([1], dtype=torch.int32, device="cuda")
    out = []
    for limit in (None, N, 3 * N):
        res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
        f = torch.empty(N, dtype=torch.float64, device="cuda")
        integ.iteration(grid, 9, 0, it, N, res, f_out=f, events_limit=limit)
        out.append((_np(res).copy(), _np(f).copy()))
    for r, f in out[1:]:
        np.testing.assert_array_equal(r, out[0][0])
        np.testing.assert_array_equal(f, out[0][1])


@pytest.mark.parametrize("prec", [0, 1])
def test_per_event_newton_outputs_do_not_depend_on_slicing(cuda, prec):
    """Per-event Newton rule: f_out and the uniforms of the sliced iteration,
    and f of the sliced integrand call, equal one slice bit for bit; the
    iteration's sums agree to rounding."""
    torch = cuda
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    N, nb, limit = 25000, 50, 6000
    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=prec,
                           newton_rule=_lib.MF_NEWTON_PER_EVENT)
    ndim = integ.n_dim
    grid = _grid(torch, ndim, nb, 3)
    it = torch.tensor([2], dtype=torch.int32, device="cuda")
    outs = []
    for lim in (None, limit):
        res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
        f = torch.empty(N, dtype=torch.float64, device="cuda")
        u = torch.empty((ndim, N), dtype=torch.float32, device="cuda")
        integ.iteration(grid, 5, 0, it, N, res, f_out=f, u_out=u, events_limit=lim)
        outs.append((_np(res).copy(), _np(f).copy(), _np(u).copy()))
    (r0, f0, u0), (r1, f1, u1) = outs
    np.testing.assert_array_equal(f1, f0)
    np.testing.assert_array_equal(u1, u0)
    assert rel_err(r1[:2], r0[:2]) < 1e-13
    assert scaled_err(r1[2:], r0[2:]) < 1e-13
    # the integrand API
    x = torch.rand((N, ndim), dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(8))
    fa = _np(integ(x))
    sliced = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=prec,
                            newton_rule=_lib.MF_NEWTON_PER_EVENT, events_limit=limit)
    np.testing.assert_array_equal(_np(sliced(x)), fa)


def test_sliced_integrand_vs_oracle(cuda, oracle):
    """mf_integrand in slices against the oracle called per slice (batch
    Newton rule per slice), FP64."""
    torch = cuda
    from madflow_gb300.vegas import FusedIntegrand

    N, limit = 3000, 700
    integ = FusedIntegrand(3, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, precision=0, events_limit=limit)
    x = np.random.default_rng(12).uniform(size=(N, integ.n_dim))
    f = _np(integ(x))
    cfg = [1, 3, 13000.0, MT, WT, 0.118, 30.0, 4.0, 0.0, 0]
    plan = oracle.TTNG(3)
    fo = np.concatenate([oracle.integrand(cfg, x[s:s + limit], plan) for s in range(0, N, limit)])
    assert scaled_err(f, fo) < 1e-12
    assert torch is not None


def test_sliced_event_output(cuda):
    """mf_vegas_events in slices (per-event Newton rule): f_out and the
    lab-frame momenta equal one slice bit for bit."""
    torch = cuda
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand, _cfg_struct

    N, nb, limit = 9000, 50, 2500
    integ = FusedIntegrand(3, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, precision=1,
                           newton_rule=_lib.MF_NEWTON_PER_EVENT)
    grid = _grid(torch, integ.n_dim, nb, 4)
    outs = []
    for lim in (0, limit):
        cs = _cfg_struct(dict(integ.cfg, events_limit=lim))
        f = torch.empty(N, dtype=torch.float64, device="cuda")
        ps = torch.empty((N, 5, 4), dtype=torch.float64, device="cuda")
        _lib.call("mf_vegas_events", integ.matrix.handle, ctypes.byref(cs), grid.data_ptr(), nb, 6, 0, 1, N,
                  f.data_ptr(), ps.data_ptr(), None)
        torch.cuda.synchronize()
        outs.append((_np(f).copy(), _np(ps).copy()))
    np.testing.assert_array_equal(outs[1][0], outs[0][0])
    np.testing.assert_array_equal(outs[1][1], outs[0][1])
    assert np.count_nonzero(outs[0][0]) > N // 4


def test_scratch_holds_two_slices(cuda):
    torch = cuda
    from madflow_gb300.vegas import FusedIntegrand

    N, limit, nb = 400_000, 50_000, 50
    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=1)
    grid = _grid(torch, integ.n_dim, nb, 5)
    it = torch.tensor([0], dtype=torch.int32, device="cuda")
    res = torch.empty(2 + integ.n_dim * nb, dtype=torch.float64, device="cuda")
    assert integ.scratch_bytes() == 0
    integ.iteration(grid, 4, 0, it, N, res, events_limit=limit)
    torch.cuda.synchronize()
    sliced = integ.scratch_bytes()
    # two buffer sets: the next slice's phase space runs beside this one's |M|^2
    assert 2 * 1700 * limit < sliced < 2 * 2100 * limit + (1 << 24)
    integ.iteration(grid, 4, 0, it, N, res)
    torch.cuda.synchronize()
    assert integ.scratch_bytes() > 1700 * N


def test_vegasflow_events_limit_fused(cuda):
    """VegasFlow(events_limit=...) on a FusedIntegrand: graph replay equals
    the eager sliced iterations bit for bit; the per-iteration sums equal a
    direct sliced iteration."""
    torch = cuda
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    N, limit = 40000, 15000
    integ = FusedIntegrand(3, kind=1, sqrts=13000.0, ptmin=30.0, etamax=4.0, precision=1)
    runs = []
    for graph in (False, True):
        v = VegasFlow(integ.n_dim, N, events_limit=limit, use_graph=graph)
        v.compile(integ)
        runs.append([v.run_event() for _ in range(3)])
    assert runs[0] == runs[1]
    # the first iteration again, directly (uniform grid, iteration 0)
    v = VegasFlow(integ.n_dim, N, events_limit=limit, use_graph=False)
    res = torch.empty(v.width, dtype=torch.float64, device="cuda")
    integ.iteration(v.grid, v.seed, v.stream_id, v.iteration, N, res, events_limit=limit)
    r = _np(res)
    n = float(N)
    est = (r[0], np.sqrt(max((n * r[1] - r[0] ** 2) / (n - 1.0), 0.0)))
    assert runs[0][0][0] == est[0] and abs(runs[0][0][1] - est[1]) <= 1e-15 * abs(est[1])


def test_negative_limit_rejected(cuda):
    torch = cuda
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand, _cfg_struct

    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
    cs = _cfg_struct(dict(integ.cfg, events_limit=-5))
    x = torch.rand((8, 100), dtype=torch.float64, device="cuda")
    f = torch.empty(100, dtype=torch.float64, device="cuda")
    st = _lib.load().mf_integrand(integ.matrix.handle, ctypes.byref(cs), x.data_ptr(), 100, f.data_ptr(), None)
    assert st == _lib.MF_ERR_ARG
    with pytest.raises(ValueError):
        FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0, events_limit=0)


@pytest.mark.parametrize("k", [2, 3])
def test_sliced_pp_channels_equal_one_slice(cuda, k):
    """p p > t t~ (j) in slices (the quark channels' buffers alternate with
    the slices too), per-event Newton rule: f_out equals one slice bit for
    bit."""
    torch = cuda
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    N, nb, limit = 30000, 50, 7000
    cuts = dict(ptmin=30.0, etamax=4.0) if k == 3 else {}
    integ = FusedIntegrand(k, kind=1, sqrts=13000.0, precision=1, initial_states="pp",
                           newton_rule=_lib.MF_NEWTON_PER_EVENT, **cuts)
    grid = _grid(torch, integ.n_dim, nb, 6)
    it = torch.tensor([1], dtype=torch.int32, device="cuda")
    outs = []
    for lim in (None, limit):
        res = torch.empty(2 + integ.n_dim * nb, dtype=torch.float64, device="cuda")
        f = torch.empty(N, dtype=torch.float64, device="cuda")
        integ.iteration(grid, 3, 0, it, N, res, f_out=f, events_limit=lim)
        outs.append((_np(res).copy(), _np(f).copy()))
    np.testing.assert_array_equal(outs[1][1], outs[0][1])
    assert rel_err(outs[1][0][:2], outs[0][0][:2]) < 1e-13
    assert np.count_nonzero(outs[0][1]) > N // 2
