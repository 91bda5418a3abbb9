"""Event output: the LHEF writer and the unweighting threshold (CPU), and
the device-side event generation and unweighting (GPU)."""
import gzip
import math
import re

import numpy as np
import pytest
import torch

from madflow_gb300 import lhe


def _parse(path):
    opener = gzip.open if str(path).endswith(".gz") else open
    text = opener(path, "rt").read()
    assert text.startswith('<LesHouchesEvents version="3.0">') and text.rstrip().endswith("</LesHouchesEvents>")
    init = re.search(r"<init>\n(.*?)</init>", text, re.S).group(1).split("\n")
    events = []
    for block in re.findall(r"<event>\n(.*?)</event>", text, re.S):
        rows = [r.split() for r in block.strip().split("\n")]
        head, parts = rows[0], rows[1:]
        assert int(head[0]) == len(parts)
        events.append((float(head[2]), np.array([[float(v) for v in p] for p in parts])))
    return init, events


def test_lhe_writer_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    p = rng.normal(size=(5, 6, 4))
    p[..., 0] = np.abs(p[..., 0]) + 10.0
    w = rng.uniform(size=5)
    path = tmp_path / "ev.lhe.gz"
    with lhe.LheWriter(path, ebeam=(6500.0, 6500.0)) as wr:
        wr.write_init(1.5, 0.01, float(w.max()))
        wr.write_events(p, w, [21, 21, 6, -6, 21, 21], 173.0, 0.118)
    init, events = _parse(path)
    assert init[0].split()[:2] == ["2212", "2212"] and init[0].split()[8] == "3"
    assert float(init[1].split()[0]) == 1.5
    assert len(events) == 5
    for e, (wt, parts) in enumerate(events):
        assert wt == pytest.approx(w[e], rel=1e-9)
        assert parts[:, 0].tolist() == [21, 21, 6, -6, 21, 21]
        assert parts[:, 1].tolist() == [-1, -1, 1, 1, 1, 1]
        np.testing.assert_allclose(parts[:, 6:9], p[e, :, 1:4], rtol=1e-9)
        np.testing.assert_allclose(parts[:, 9], p[e, :, 0], rtol=1e-9)


def test_lhe_dynamic_scale_per_event(tmp_path):
    """Events of a dynamic-scale run carry their own scale and alpha_s:
    mu = sum of the outgoing m_T / 2 and alpha_s(mu^2) at one loop from
    alpha_s(M_Z^2) (scripts/madflow_exec.py:428-431)."""
    rng = np.random.default_rng(3)
    p = np.zeros((4, 4, 4))
    p[:, 2:, 1:] = rng.normal(scale=100.0, size=(4, 2, 3))
    p[:, 2:, 0] = np.sqrt(173.0**2 + (p[:, 2:, 1:] ** 2).sum(-1))
    mu, a = lhe.dynamic_scale(p, 0.118)
    mt = np.sqrt(173.0**2 + p[:, 2:, 1] ** 2 + p[:, 2:, 2] ** 2)
    np.testing.assert_allclose(mu, mt.sum(-1) / 2.0, rtol=1e-14)
    b0 = 23.0 / (12.0 * math.pi)
    np.testing.assert_allclose(a, 0.118 / (1.0 + 0.118 * b0 * np.log(mu**2 / 91.1876**2)), rtol=1e-14)
    assert np.all(a < 0.118)  # mu >= mt > M_Z
    path = tmp_path / "dyn.lhe"
    with lhe.LheWriter(path, ebeam=(6500.0, 6500.0)) as wr:
        wr.write_init(1.0, 0.1, 1.0)
        wr.write_events(p, np.ones(4), [21, 21, 6, -6], mu, a)
    heads = [line.split() for line in open(path).read().split("<event>\n")[1:]]
    np.testing.assert_allclose([float(h[3]) for h in heads], mu, rtol=1e-9)
    np.testing.assert_allclose([float(h[5]) for h in heads], a, rtol=1e-9)


def test_truncated_wmax():
    w = torch.tensor(np.random.default_rng(2).pareto(1.5, size=5000))
    assert lhe.truncated_wmax(w, 0.0) == float(w.max())
    t = lhe.truncated_wmax(w, 0.01)
    a = w.abs()
    assert float(torch.clamp(a - t, min=0).sum()) <= 0.01 * float(a.sum()) * (1 + 1e-12)
    # the next smaller distinct weight would truncate more than the allowed fraction
    s = torch.sort(a, descending=True).values
    nxt = s[s < t].max()
    assert float(torch.clamp(a - nxt, min=0).sum()) > 0.01 * float(a.sum())


@pytest.mark.gpu
def test_unweight_device(cuda):
    w = torch.tensor(np.random.default_rng(3).uniform(size=200_000) ** 4, device="cuda")
    wmax = 0.5
    idx, rel = lhe.unweight(w, wmax, seed=5, stream_id=1)
    idx2, _ = lhe.unweight(w, wmax, seed=5, stream_id=1)
    assert torch.equal(idx, idx2)
    expect = float(torch.clamp(w / wmax, max=1.0).sum())
    assert abs(idx.numel() - expect) < 5 * math.sqrt(expect)
    assert float(rel.min()) >= 1.0
    over = w[idx] > wmax
    assert torch.allclose(rel[over], w[idx][over] / wmax)


@pytest.mark.gpu
def test_event_generation_ggttx(cuda, tmp_path):
    """Unweighted gg > tt~ events at fixed sqrt(s): lab = c.o.m. momenta that
    conserve momentum, on-shell tops, the f of the events path equal to the
    fused iteration's, and an LHE file that reads back."""
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
    v = VegasFlow(8, 50_000, use_graph=False)
    v.compile(integ)
    v.run_integration(3)
    n = 20_000
    f = torch.empty(n, dtype=torch.float64, device="cuda")
    ps = torch.empty((n, 4, 4), dtype=torch.float64, device="cuda")
    import ctypes

    from madflow_gb300.config import stream_ptr

    _lib.call("mf_vegas_events", integ.matrix.handle, ctypes.byref(integ._cs), v.grid.data_ptr(), v.nbins, 123, 0, 0,
              n, f.data_ptr(), ps.data_ptr(), stream_ptr())
    f_it = torch.empty(n, dtype=torch.float64, device="cuda")
    res = torch.empty(2 + 8 * v.nbins, dtype=torch.float64, device="cuda")
    it = torch.zeros(1, dtype=torch.int32, device="cuda")
    integ.iteration(v.grid, 123, 0, it, n, res, f_out=f_it)
    assert torch.equal(f, f_it)
    p = ps.cpu().numpy()
    tot = p[:, 2:].sum(axis=1) - p[:, :2].sum(axis=1)
    assert np.abs(tot).max() < 1e-9 * 1000.0
    m2 = p[:, 2, 0] ** 2 - (p[:, 2, 1:] ** 2).sum(-1)
    np.testing.assert_allclose(np.sqrt(m2), 173.0, rtol=1e-7)
    stats = lhe.generate_events(integ, v, 2000, tmp_path / "gg_ttx.lhe.gz", batch=100_000, trunc=1e-3)
    assert stats["kept"] == 2000
    init, events = _parse(tmp_path / "gg_ttx.lhe.gz")
    assert len(events) == 2000
    assert sum(e[0] for e in events) == pytest.approx(stats["xsec_pb"], rel=1e-6)
    assert abs(stats["xsec_pb"] - v.history[-1][0]) < 5 * math.hypot(stats["xerr_pb"], v.history[-1][1])


@pytest.mark.gpu
def test_event_generation_dynamic_scale(cuda, tmp_path):
    """Hadronic g g > t t~ at madflow's dynamical scale: the unweighted
    events carry their own mu (sum of the outgoing m_T / 2 of the written
    momenta) and alpha_s(mu^2), and the file's cross section agrees with the
    VEGAS integral of the same integrand."""
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    integ = FusedIntegrand(2, kind=1, sqrts=13000.0, q2="dynamic", precision=0)
    v = VegasFlow(integ.n_dim, 100_000, use_graph=False)
    v.compile(integ)
    v.run_integration(4)
    path = tmp_path / "gg_ttx_dyn.lhe"
    stats = lhe.generate_events(integ, v, 500, path, batch=100_000, trunc=1e-3)
    assert stats["kept"] == 500
    text = open(path).read()
    heads = [blk.split("\n")[0].split() for blk in text.split("<event>\n")[1:]]
    _, events = _parse(path)
    p = np.stack([parts[:, [9, 6, 7, 8]] for _, parts in events])  # (E, px, py, pz)
    mu, a = lhe.dynamic_scale(p, 0.118)
    np.testing.assert_allclose([float(h[3]) for h in heads], mu, rtol=1e-8)
    np.testing.assert_allclose([float(h[5]) for h in heads], a, rtol=1e-8)
    assert np.all(mu >= 173.0 * (1 - 1e-9)) and np.all(a < 0.118)
    assert abs(stats["xsec_pb"] - v.history[-1][0]) < 5 * math.hypot(stats["xerr_pb"], v.history[-1][1])
