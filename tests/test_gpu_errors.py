"""Error paths of the CUDA library, exercised without a GPU fault.

* A bounded wait on the tensor cores that runs out: the wait limit of a
  handle is set to 0 tries, so the first wait of every thread block gives up
  at once (the block still drains its tensor-core work at the normal limit
  before freeing its tensor memory).  Every event that needed work must come
  out NaN, error bit 0 must be raised, and the handle must work normally once
  the limit is restored.
* Non-finite caller input (NaN / inf momenta or points): the affected events
  give NaN |M|^2 (mf_smatrix) or are counted and zeroed in the weights
  (mf_integrand, VEGAS); no other event changes.
* Caller bin indices outside [0, nbins) in mf_vegas_accumulate add to no bin.
"""
import ctypes
import warnings

import numpy as np
import pytest

from conftest import GC10, GC11, GC12, MT, WT

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _flags(handle, clear=1):
    from madflow_gb300 import _lib

    f = ctypes.c_int()
    _lib.call("mf_process_error_flags", handle, ctypes.byref(f), clear)
    return f.value


def _points(oracle, k, n, seed):
    x = np.random.default_rng(seed).uniform(size=(n, 4 * k + 2))
    p, *_ = oracle.ramboflow(x, k + 2, 13000.0, [MT, MT] + [0.0] * (k - 2))
    return p


@pytest.mark.parametrize("k,n", [(4, 3000), (5, 400)])
def test_tensor_core_timeout_gives_nan_for_every_event(cuda, oracle, k, n):
    """More events than blocks, so every block meets the error on its first
    event and must mark its later ones too."""
    from madflow_gb300 import _lib
    from madflow_gb300.matrix import PROCESSES

    m = PROCESSES[k](precision=1)
    m.set_tuning(1, 1)  # tensor-core colour sum, one wave
    p = _points(oracle, k, n, 70 + k)
    _flags(m.handle)
    good = _np(m.smatrix(p, MT, WT, GC10, GC11, GC12))
    assert np.all(np.isfinite(good)) and _flags(m.handle) == 0
    _lib.call("mf_process_set_wait_limit", m.handle, 0)
    bad = _np(m.smatrix(p, MT, WT, GC10, GC11, GC12))
    assert np.all(np.isnan(bad)), f"{int(np.sum(~np.isnan(bad)))} events kept a value"
    assert _flags(m.handle) & 1
    # the per-helicity outputs of the affected events are NaN as well, but
    # for the first event of each block (its colour sums per helicity come
    # from the SIMT lanes): rows of events beyond the grid are all NaN
    tot, hel = m.smatrix_per_helicity(p, MT, WT, GC10, GC11, GC12)
    assert np.all(np.isnan(_np(tot)))
    grid = int(np.sum(np.isfinite(_np(hel)).all(axis=0)))
    assert np.all(np.isnan(_np(hel)[:, -50:])) and grid < n
    assert _flags(m.handle) & 1
    # the context and the handle stay usable
    _lib.call("mf_process_set_wait_limit", m.handle, 1000)
    again = _np(m.smatrix(p, MT, WT, GC10, GC11, GC12))
    assert _flags(m.handle) == 0
    np.testing.assert_array_equal(again, good)


def test_tensor_core_timeout_raises_in_vegas(cuda):
    """The fused iteration with the wait limit at 0: the passing events get
    NaN, the accumulation zeroes and counts them, and VegasFlow raises on
    the device error flag when it reads the iteration's result; events that
    fail the cuts needed no work and stay 0."""
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=1)
    _lib.call("mf_process_set_tuning", integ.matrix.handle, 1, 1)
    integ.set_wait_limit(0)
    x = torch.rand((5000, integ.n_dim), dtype=torch.float64, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(3))
    f = _np(integ(x))
    assert np.all(f == 0)  # NaN weights of the passing events were zeroed
    with pytest.raises(_lib.DeviceError):
        integ.check_errors()
    v = VegasFlow(integ.n_dim, 20000, use_graph=False)
    v.compile(integ)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        with pytest.raises(_lib.DeviceError):
            v.run_event()
    integ.set_wait_limit(1000)
    integ.check_errors()
    fg = _np(integ(x))
    assert np.all(np.isfinite(fg)) and np.count_nonzero(fg) > 1000
    assert integ.check_errors() == 0


@pytest.mark.parametrize("k,prec", [(2, 0), (2, 1), (3, 1), (4, 0), (4, 1)])
def test_nonfinite_momenta_smatrix(cuda, oracle, k, prec):
    """NaN or inf momenta give NaN |M|^2 for their own events only (several
    events share a block for two and three gluons)."""
    from madflow_gb300.matrix import PROCESSES

    m = PROCESSES[k](precision=prec)
    p = _points(oracle, k, 500, 80 + k)
    clean = _np(m.smatrix(p, MT, WT, GC10, GC11, GC12))
    q = p.copy()
    bad = np.array([0, 7, 8, 250, 499])
    q[bad[:3], 2, 0] = np.nan
    q[bad[3], 4 if k > 2 else 1, 3] = np.inf
    q[bad[4], 0, 0] = -np.inf
    out = _np(m.smatrix(q, MT, WT, GC10, GC11, GC12))
    assert np.all(~np.isfinite(out[bad]))
    keep = np.setdiff1d(np.arange(len(p)), bad)
    np.testing.assert_array_equal(out[keep], clean[keep])


@pytest.mark.parametrize("prec", [0, 1])
def test_nonfinite_points_integrand(cuda, prec):
    """Non-finite points of mf_integrand: their weights are counted and
    zeroed, and they take no part in the batch Newton rule, so every other
    event is bit-identical to a clean call."""
    import torch

    from madflow_gb300.vegas import FusedIntegrand

    for integ in (FusedIntegrand(2, kind=0, sqrts=1000.0, precision=prec),
                  FusedIntegrand(4, kind=1, sqrts=13000.0, precision=prec)):
        x = torch.rand((4000, integ.n_dim), dtype=torch.float64, device="cuda",
                       generator=torch.Generator(device="cuda").manual_seed(11))
        integ.check_errors()
        clean = _np(integ(x))
        assert integ.check_errors() == 0
        bad = torch.tensor([3, 4, 1000, 3999], device="cuda")
        y = x.clone()
        y[bad, 0] = float("nan")
        y[bad[-1], 1] = float("inf")
        f = _np(integ(y))
        assert integ.check_errors() == len(bad)
        b = _np(bad)
        assert np.all(f[b] == 0)
        keep = np.setdiff1d(np.arange(len(f)), b)
        np.testing.assert_array_equal(f[keep], clean[keep])


def test_nonfinite_python_integrand_counted(cuda):
    """The generic (callable) VEGAS path counts and zeroes non-finite values
    of the caller's integrand and warns."""
    import torch

    from madflow_gb300.vegas import VegasFlow

    def f(x, n_dim=None, weight=None):
        y = torch.ones(x.shape[0], dtype=torch.float64, device=x.device)
        y[::100] = float("nan")
        return y

    v = VegasFlow(3, 1000, use_graph=False)
    v.compile(f)
    with pytest.warns(RuntimeWarning, match="non-finite"):
        res, err = v.run_event()
    assert v.nonfinite == 10
    assert abs(res - 0.99) < 1e-12


def test_accumulate_ignores_out_of_range_bins(cuda, oracle):
    import torch

    from madflow_gb300 import _lib

    rng = np.random.default_rng(9)
    ndim, nb, N = 4, 50, 3000
    bins = rng.integers(0, nb, size=(N, ndim)).astype(np.int32)
    bins[::7, 1] = -1
    bins[::11, 2] = nb
    bins[5, 3] = 1 << 30
    fw = rng.exponential(size=N)
    fw_d = torch.tensor(fw, device="cuda")
    jac_d = torch.ones(N, dtype=torch.float64, device="cuda")
    bins_d = torch.tensor(bins.T.copy(), device="cuda")
    for fn in ("mf_vegas_accumulate", "mf_vegas_accumulate_noalloc"):
        res = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
        _lib.call(fn, fw_d.data_ptr(), jac_d.data_ptr(), bins_d.data_ptr(), N, ndim, nb, 1.0, res.data_ptr(), None)
        torch.cuda.synchronize()
        r = _np(res)
        hist = np.zeros((ndim, nb))
        for d in range(ndim):
            ok = (bins[:, d] >= 0) & (bins[:, d] < nb)
            np.add.at(hist[d], bins[ok, d], fw[ok] ** 2)
        assert abs(r[0] / fw.sum() - 1) < 1e-12 and abs(r[1] / (fw ** 2).sum() - 1) < 1e-12
        np.testing.assert_allclose(r[2:].reshape(ndim, nb), hist, rtol=1e-12, atol=0)
