"""Sharded integration: the one exchange per iteration (sum of the results
vector over the ranks) and the estimate from the summed sums, on gloo ranks
on the CPU; the sharded VegasFlow path on one GPU."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from madflow_gb300.vegas import iteration_estimate, reduce_results

NDIM, NB, N = 3, 5, 4000


def _rank_results(rank):
    """A results vector of one rank from synthetic weights (w = f jac / n)."""
    rng = np.random.default_rng(100 + rank)
    fj = rng.exponential(size=N)
    bins = rng.integers(0, NB, size=(NDIM, N))
    w = fj / N
    out = np.zeros(2 + NDIM * NB)
    out[0], out[1] = w.sum(), (w * w).sum()
    for d in range(NDIM):
        np.add.at(out[2 + d * NB: 2 + (d + 1) * NB], bins[d], w * w)
    return fj, out


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    _, r = _rank_results(rank)
    t = torch.tensor(r)
    reduce_results(t)
    q.put((rank, t.numpy().copy()))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_sums_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank holds the same summed vector, equal to the sum of the parts
    parts = [_rank_results(r) for r in range(world)]
    want = sum(p[1] for p in parts)
    for r in range(world):
        np.testing.assert_allclose(got[r], want, rtol=1e-14)
    # the estimate from the summed sums is the mean and error of all events
    fj = np.concatenate([p[0] for p in parts])
    res, sig = iteration_estimate(want[0], want[1], N, world)
    assert res == pytest.approx(fj.mean(), rel=1e-12)
    assert sig == pytest.approx(fj.std(ddof=1) / np.sqrt(fj.size), rel=1e-9)


def test_single_rank_estimate_matches_unsharded():
    fj, r = _rank_results(0)
    res, sig = iteration_estimate(r[0], r[1], N, 1)
    n = float(N)
    assert res == pytest.approx(r[0])
    assert sig == pytest.approx(np.sqrt((n * r[1] - r[0] ** 2) / (n - 1.0)), rel=1e-12)


@pytest.mark.gpu
def test_sharded_vegasflow_one_rank(cuda):
    """A group of one rank gives the unsharded integration bit for bit."""
    from madflow_gb300.vegas import FusedIntegrand, VegasFlow

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    os.environ.setdefault("MASTER_PORT", str(_free_port()))
    dist.init_process_group("gloo", rank=0, world_size=1)
    try:
        integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
        a = VegasFlow(8, 20000, use_graph=False)
        a.compile(integ)
        ra = a.run_integration(3)
        b = VegasFlow(8, 20000, use_graph=False, process_group=dist.group.WORLD)
        b.compile(integ)
        rb = b.run_integration(3)
        assert ra == rb
        assert torch.equal(a.grid, b.grid)
    finally:
        dist.destroy_process_group()


# ---- VegasFlow(process_group=...) end to end on two gloo ranks ------------------
# The orchestration of a sharded integration runs as in production (stream id
# per rank, one all-reduce of the results vector per iteration, refinement on
# every rank, the estimate from the summed sums); the fused GPU iteration and
# the refinement are replaced by their CPU restatements from the oracle.
SH_NDIM, SH_NB, SH_N, SH_ITERS = 4, 10, 3000, 3


def _stub_f(x):
    return np.exp(-30.0 * ((x - 0.4) ** 2).sum(axis=1)) + 0.1


def _stub_results(grid, seed, stream_id, it, n):
    import oracle

    u = oracle.uniforms(seed, stream_id, it, 0, n, SH_NDIM)
    x, jac, bins = oracle.vegas_sample(grid, u)
    sums, hist = oracle.vegas_accumulate(_stub_f(x) * jac / n, bins, SH_NB)
    return np.concatenate([sums, hist.ravel()])


def _cpu_vegasflow(group):
    """A VegasFlow whose device work runs on the CPU (see above)."""
    import madflow_gb300.vegas as V
    import oracle

    class Stub(V.FusedIntegrand):
        def __init__(self):
            self.n_dim = SH_NDIM

        def iteration(self, grid, seed, stream_id, iteration_dev, n_events, results, f_out=None, u_out=None,
                      events_limit=None):
            r = _stub_results(grid.numpy(), seed, stream_id, int(iteration_dev.item()), n_events)
            results.copy_(torch.tensor(r))

        def check_errors(self, clear=True):
            return 0

    def refine(self):
        g = oracle.vegas_refine(self.grid.numpy(), self.results[2:].reshape(self.n_dim, self.nbins).numpy(),
                                self.alpha)
        self.grid.copy_(torch.tensor(g))

    V.device = lambda: torch.device("cpu")
    V.VegasFlow._refine = refine
    v = V.VegasFlow(SH_NDIM, SH_N, nbins=SH_NB, seed=4, process_group=group, use_graph=False)
    v.compile(Stub())
    return v


def _vegas_worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    v = _cpu_vegasflow(dist.group.WORLD)
    per_iter = [v.run_event() for _ in range(SH_ITERS)]
    q.put((rank, v.stream_id, per_iter, v.grid.numpy().copy()))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_vegasflow_gloo_two_ranks():
    import oracle

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_vegas_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(world):
        rank, sid, per_iter, grid = q.get(timeout=180)
        got[rank] = (sid, per_iter, grid)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # each rank draws its own Philox stream
    assert [got[r][0] for r in range(world)] == [0, 1]
    # both ranks hold the same estimates and the same refined grid
    assert got[0][1] == got[1][1]
    np.testing.assert_array_equal(got[0][2], got[1][2])
    # one process running both streams gives the same
    grid = np.tile(np.linspace(0.0, 1.0, SH_NB + 1), (SH_NDIM, 1))
    for it in range(SH_ITERS):
        r = sum(_stub_results(grid, 4, s, it, SH_N) for s in range(world))
        want = iteration_estimate(r[0], r[1], SH_N, world)
        assert got[0][1][it][0] == pytest.approx(want[0], rel=1e-12)
        assert got[0][1][it][1] == pytest.approx(want[1], rel=1e-9)
        grid = oracle.vegas_refine(grid, r[2:].reshape(SH_NDIM, SH_NB), 1.5)
    np.testing.assert_allclose(got[0][2], grid, rtol=1e-13, atol=1e-15)
