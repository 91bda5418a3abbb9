"""The CUDA piecewise-quadratic coupling kernels against a plain PyTorch FP64
restatement of the same transform (forward, inverse, log-Jacobian, gradients),
and the flow sampler's density against its own inverse.  Tolerances: 2e-4
absolute on values in [0,1] and 1e-3 relative on gradients (FP32 kernels with
fast exp/log)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_pq(x, params, K):
    """Reference piecewise-quadratic CDF and log pdf (float64, autograd)."""
    import torch

    Wt, Vt = params[..., :K], params[..., K:]
    W = torch.softmax(Wt, dim=-1)
    E = torch.exp(Vt - Vt.max(dim=-1, keepdim=True).values)
    norm = (0.5 * (E[..., :-1] + E[..., 1:]) * W).sum(-1, keepdim=True)
    V = E / norm
    edges = torch.cat([torch.zeros_like(W[..., :1]), torch.cumsum(W, -1)], -1)
    cdf = torch.cat([torch.zeros_like(W[..., :1]), torch.cumsum(0.5 * (V[..., :-1] + V[..., 1:]) * W, -1)], -1)
    b = (x.unsqueeze(-1) >= edges[..., 1:K]).sum(-1, keepdim=True)
    e_b = edges.gather(-1, b)
    c_b = cdf.gather(-1, b)
    W_b = W.gather(-1, b)
    V_b = V.gather(-1, b)
    V_b1 = V.gather(-1, b + 1)
    t = x.unsqueeze(-1) - e_b
    D = V_b1 - V_b
    y = c_b + t * V_b + 0.5 * t * t / W_b * D
    pdf = V_b + t / W_b * D
    return y.squeeze(-1), torch.log(pdf.squeeze(-1)).sum(-1)


@pytest.fixture
def batch(cuda):
    import torch

    g = torch.Generator(device="cuda").manual_seed(0)
    n, nb, K = 4096, 9, 16
    x = torch.rand((n, nb), generator=g, device="cuda")
    params = torch.randn((n, nb, 2 * K + 1), generator=g, device="cuda")
    return x, params, K


def test_pq_forward_and_backward(batch):
    import torch

    from madflow_gb300.flow import pq_forward

    x, params, K = batch
    xr = x.double().requires_grad_(True)
    pr = params.double().requires_grad_(True)
    yr, ldr = torch_pq(xr, pr, K)
    xk = x.clone().requires_grad_(True)
    pk = params.clone().requires_grad_(True)
    yk, ldk = pq_forward(xk, pk, K)
    assert torch.max(torch.abs(yk.double() - yr)).item() < 2e-5
    assert torch.max(torch.abs(ldk.double() - ldr) / (1 + ldr.abs())).item() < 2e-4
    gy = torch.randn_like(yr)
    gl = torch.randn_like(ldr)
    torch.autograd.backward([yr, ldr], [gy, gl])
    torch.autograd.backward([yk, ldk], [gy.float(), gl.float()])
    for a, b in ((xk.grad, xr.grad), (pk.grad, pr.grad)):
        err = torch.max(torch.abs(a.double() - b)) / torch.max(torch.abs(b))
        assert err.item() < 1e-3


def test_pq_inverse_roundtrip(batch):
    import torch

    from madflow_gb300.flow import pq_forward, pq_inverse

    x, params, K = batch
    with torch.no_grad():
        y, ld = pq_forward(x, params, K)
        x2, ld2 = pq_inverse(y, params, K)
    assert torch.max(torch.abs(x2 - x)).item() < 2e-4
    assert torch.max(torch.abs(ld2 - ld) / (1 + ld.abs())).item() < 2e-3


def test_flow_density_consistent_and_normalised(cuda):
    import torch

    from madflow_gb300.flow import NormalizingFlow

    flow = NormalizingFlow(6, n_layers=4, bins=8, hidden=32, seed=3, bf16=False)
    with torch.no_grad():
        for p in flow.parameters():
            p.add_(0.3 * torch.randn_like(p))
        x, logq = flow.sample(200_000, seed=5)
        lp = flow.log_prob(x)
    assert torch.max(torch.abs(lp.double() - logq)).item() < 2e-3
    # E_q[1/q] = volume of the unit hypercube = 1
    v = torch.exp(-logq).mean().item()
    assert abs(v - 1.0) < 0.02


def test_flow_training_reduces_variance(cuda):
    import torch

    from madflow_gb300.flow import NormalizingFlow, train_flow

    def peaked(x):  # a narrow Gaussian bump in 4 dimensions
        return torch.exp(-(((x - 0.3) / 0.08) ** 2).sum(-1))

    flow = NormalizingFlow(4, n_layers=4, bins=16, hidden=64, seed=1)
    hist = train_flow(flow, peaked, n_batches=12, batch_size=100_000, minibatch=25_000, lr=5e-3)
    assert hist[-1] < 0.5 * hist[0]


@pytest.mark.parametrize("resample", [0, 20_000])
def test_adaptive_flow_integration(cuda, resample):
    """Training batches double as estimates: the combined result of a
    normalised bump agrees with its integral within the quoted error, and the
    quoted error reaches the target (training on all events, or on events
    resampled with probability w^2)."""
    import math

    import torch

    from madflow_gb300.flow import NormalizingFlow, adaptive_flow_integration

    sig = 0.1
    norm = (sig * math.sqrt(math.pi) * math.erf(0.5 / sig)) ** 3  # integral over the unit cube

    def bump(x):
        return torch.exp(-(((x - 0.5) / sig) ** 2).sum(-1)) / norm

    flow = NormalizingFlow(3, n_layers=4, bins=16, hidden=32, seed=2)
    res, err, info = adaptive_flow_integration(flow, bump, target_rel_error=3e-3, batch_size=50_000,
                                               max_batches=60, train_batches=20, minibatch=10_000 if resample else 25_000,
                                               lr=5e-3, resample=resample)
    assert err / res <= 3e-3
    assert abs(res - 1.0) < 4 * err
    assert info["batches"] <= 60


def test_adaptive_flow_on_vegas_grid(cuda):
    """The flow on top of an adapted VEGAS grid: the weights carry the grid
    jacobian, so the estimate of a normalised bump stays unbiased."""
    import math

    import torch

    from madflow_gb300.flow import NormalizingFlow, adaptive_flow_integration
    from madflow_gb300.vegas import VegasFlow

    sig = 0.1
    norm = (sig * math.sqrt(math.pi) * math.erf(0.5 / sig)) ** 3

    def bump(x, n_dim=None, weight=None):
        return torch.exp(-(((x - 0.5) / sig) ** 2).sum(-1)) / norm

    v = VegasFlow(3, 100_000, seed=3, use_graph=False)
    v.compile(bump)
    r0, e0 = v.run_integration(4)
    flow = NormalizingFlow(3, n_layers=4, bins=16, hidden=32, seed=2)
    res, err, info = adaptive_flow_integration(flow, bump, target_rel_error=2e-3, batch_size=50_000, max_batches=60,
                                               train_batches=10, minibatch=25_000, lr=3e-3, grid=v.grid,
                                               prior=(1.0 / e0**2, r0 / e0**2))
    assert err / res <= 2e-3
    assert abs(res - 1.0) < 4 * err


@pytest.mark.parametrize("dim,bins", [(18, 8), (18, 4), (7, 16), (18, 16), (32, 8)])
def test_fused_tensor_core_sampling(cuda, dim, bins):
    """mf_flow_inv_layer_tc (conditioner MLP as three tcgen05 TF32 GEMMs and
    the inverse transform in one kernel per layer) against the layer-by-layer
    path with FP32 GEMMs (cuBLAS) and the separate inverse kernel, on the
    same uniforms and random weights (every layer, the last included, so the
    map is far from the identity).  The MLP inputs and weights are rounded to
    TF32 (10-bit mantissa) in the fused kernel: points agree to 2e-3 and
    log-densities to 2e-2 absolute; and the fused sampler's log density is
    its map's own (against the FP32 forward log_prob, same tolerance).
    (18, 16) and (32, 8) have more than 256 MLP outputs per layer (297, 272):
    the third GEMM runs in two column chunks."""
    import torch

    from madflow_gb300.flow import NormalizingFlow

    torch.manual_seed(3)
    f = NormalizingFlow(dim, n_layers=4, bins=bins, hidden=64, n_hidden=2, seed=1, bf16=False, tf32=True, fused=True)
    with torch.no_grad():
        for p in f.parameters():
            p.copy_(torch.randn_like(p) * (0.5 / max(1, p.shape[-1]) ** 0.5))
    g = NormalizingFlow(dim, n_layers=4, bins=bins, hidden=64, n_hidden=2, seed=1, bf16=False, tf32=False,
                        fused=False, native=False)
    g.load_state_dict(f.state_dict())
    assert f.fused and not g.fused
    n = 100_003  # not a multiple of the 128-point tile
    zf, lf = f.sample(n, seed=11, iteration=2)
    zg, lg = g.sample(n, seed=11, iteration=2)
    assert zf.shape == (n, dim) and torch.isfinite(zf).all() and torch.isfinite(lf).all()
    assert float((zf - zg).abs().max()) < 2e-3
    assert float((lf - lg).abs().max()) < 2e-2
    with torch.no_grad():
        lp = g.log_prob(zf.float())
    assert float((lp.double() - lf).abs().max()) < 2e-2


@pytest.mark.parametrize("dim,bins", [(18, 16), (18, 8), (7, 4), (32, 8)])
def test_fused_bf16_sampling(cuda, dim, bins):
    """mf_flow_inv_layer_tc_bf16 (the three MLP GEMMs on BF16 operands with
    FP32 accumulation, tcgen05 kind::f16) against a PyTorch restatement that
    rounds the same operands to BF16 (inputs 2z - 1, weights, hidden
    activations after bias and ReLU) and multiplies in FP32, followed by the
    inverse transform kernel: points within 2e-3, log-densities within 2e-2
    (the two differ only in the FP32 summation order and, rarely, a hidden
    activation that rounds to the other BF16 neighbour).  And the sampler's
    log density is its own map's: E_q[1/q] = 1 over the unit hypercube."""
    import torch

    from madflow_gb300.flow import NormalizingFlow, pq_inverse

    torch.manual_seed(4)
    f = NormalizingFlow(dim, n_layers=4, bins=bins, hidden=64, n_hidden=2, seed=2, tc_bf16=True)
    with torch.no_grad():
        for p in f.parameters():
            p.copy_(torch.randn_like(p) * (0.5 / max(1, p.shape[-1]) ** 0.5))
    assert f.fused and f.tc_bf16
    n = 100_003  # not a multiple of the 128-point tile
    zf, lf = f.sample(n, seed=13, iteration=1)
    assert zf.shape == (n, dim) and torch.isfinite(zf).all() and torch.isfinite(lf).all()

    def bf(t):
        return t.bfloat16().float()

    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        with torch.no_grad():
            u = torch.empty((dim, n), dtype=torch.float64, device="cuda")
            from madflow_gb300 import _lib
            from madflow_gb300.config import stream_ptr

            _lib.call("mf_philox_uniforms", 13, 7, 1, 0, n, dim, u.data_ptr(), stream_ptr())
            z = u.T.float().contiguous()
            lq = torch.zeros(n, dtype=torch.float64, device="cuda")
            for l, net in enumerate(f.nets):
                ib, ia = f._idx[l]
                h1 = torch.relu(bf(2.0 * z[:, ia] - 1.0) @ bf(net[0].weight).T + net[0].bias)
                h2 = torch.relu(bf(h1) @ bf(net[2].weight).T + net[2].bias)
                par = (bf(h2) @ bf(net[4].weight).T + net[4].bias).reshape(n, len(ib), 2 * bins + 1)
                xb, ld = pq_inverse(z[:, ib].contiguous(), par.contiguous(), bins)
                z[:, ib] = xb
                lq += ld.double()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    assert float((zf - z.double()).abs().max()) < 2e-3
    assert float((lf - lq).abs().max()) < 2e-2
    w = torch.exp(-lf)
    v, se = w.mean().item(), (w.std() / n**0.5).item()
    assert abs(v - 1.0) < 5 * se + 1e-3, (v, se)


def test_graphed_training_step_matches_eager(cuda):
    """The training step captured as a CUDA graph (log-density, backward,
    Adam) moves the weights as the eager step does, and leaves them untouched
    when it is built (the capture's warm-up steps are undone)."""
    import torch

    from madflow_gb300.flow import NormalizingFlow, _GraphedStep, _train_step

    a = NormalizingFlow(6, n_layers=4, bins=8, hidden=32, seed=5, bf16=False, tf32=False)
    b = NormalizingFlow(6, n_layers=4, bins=8, hidden=32, seed=5, bf16=False, tf32=False)
    b.load_state_dict(a.state_dict())
    oa = torch.optim.Adam(a.parameters(), lr=1e-2)
    ob = torch.optim.Adam(b.parameters(), lr=1e-2, capturable=True)
    step = _GraphedStep(b, ob, 4096)
    for pa, pb in zip(a.parameters(), b.parameters()):
        assert torch.equal(pa, pb)
    g = torch.Generator(device="cuda").manual_seed(1)
    for it in range(4):
        x = torch.rand((20_000, 6), device="cuda", dtype=torch.float64, generator=g)
        w = torch.exp(-((x - 0.3) ** 2).sum(-1) * 8.0)
        torch.manual_seed(10 + it)
        _train_step(a, oa, x, w, 8192, resample=4096)
        torch.manual_seed(10 + it)
        _train_step(b, ob, x, w, 8192, resample=4096, step=step)
    with torch.no_grad():
        for pa, pb in zip(a.parameters(), b.parameters()):
            assert float((pa - pb).abs().max()) < 1e-5
        assert any(float(p.abs().max()) > 0 for p in list(b.parameters())[-2:])


def _fp64_logq(flow, x):
    """log q(x) of the flow in FP64 torch autograd: every layer's MLP with the
    flow's weights in float64 and the transform of torch_pq above."""
    import torch

    z = x.double()
    logq = torch.zeros(x.shape[0], dtype=torch.float64, device=x.device)
    for l in reversed(range(len(flow.masks))):
        ib, ia = flow._idx[l]
        net = flow.nets[l]
        h = 2.0 * z[:, ia] - 1.0
        for i in (0, 2, 4):
            lin = net[i]
            h = h @ lin.weight.double().t() + lin.bias.double()
            if i < 4:
                h = torch.relu(h)
        params = h.reshape(-1, len(ib), 2 * flow.K + 1)
        y, ld = torch_pq(z[:, ib].clamp(0.0, 1.0), params, flow.K)
        z = z.index_copy(1, ib, y)
        logq = logq + ld
    return logq


def _random_flow(dim, bins, seed):
    import torch

    from madflow_gb300.flow import NormalizingFlow

    f = NormalizingFlow(dim, n_layers=6, bins=bins, hidden=64, n_hidden=2, seed=seed)
    assert f.native
    torch.manual_seed(seed)
    with torch.no_grad():
        for p in f.parameters():  # every layer, the last included: far from the identity map
            p.copy_(torch.randn_like(p) * (0.6 / max(1, p.shape[-1]) ** 0.5))
    return f


@pytest.mark.parametrize("dim,bins", [(18, 16), (18, 8), (7, 4)])
def test_native_density_matches_fp64(cuda, dim, bins):
    """The hand-written density-direction layer kernels (MLP + transform)
    against FP64 torch: log q within 2e-3 absolute."""
    import torch

    f = _random_flow(dim, bins, 7)
    x = torch.rand((3001, dim), device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    lq = f.native_log_prob(x)
    ref = _fp64_logq(f, x)
    assert float((lq.detach().double() - ref.detach()).abs().max()) < 2e-3


@pytest.mark.parametrize("dim,bins", [(18, 16), (7, 4)])
def test_native_gradient_matches_fp64_autograd(cuda, dim, bins):
    """The hand-written gradient kernels (transform backward + MLP backward
    as tiled GEMMs, fixed-order block sums) against FP64 torch autograd of
    L = sum_i c_i log q(x_i), per weight tensor within 2e-3 of its largest
    entry; 1001 points (not a multiple of the 32-point tile).  The same call
    twice gives bit-identical gradients."""
    import torch

    f = _random_flow(dim, bins, 11)
    n = 1001
    g = torch.Generator(device="cuda").manual_seed(4)
    x = torch.rand((n, dim), device="cuda", generator=g)
    c = torch.randn(n, device="cuda", generator=g) / n
    lq = f.native_backward(x, c)
    got = [p.grad.clone() for p in f.parameters()]
    f.native_backward(x, c)
    for a, p in zip(got, f.parameters()):
        assert torch.equal(a, p.grad)
    params64 = [p.detach().double().requires_grad_(True) for p in f.parameters()]
    with torch.no_grad():
        saved = [p.detach().clone() for p in f.parameters()]
    # the FP64 forward rebuilt with float64 copies of the weights
    def fp64_logq(ps):
        z = x.double()
        out = torch.zeros(n, dtype=torch.float64, device=x.device)
        it = iter(ps)
        layers = [[next(it) for _ in range(6)] for _ in range(len(f.masks))]
        for l in reversed(range(len(f.masks))):
            ib, ia = f._idx[l]
            W1, b1, W2, b2, W3, b3 = layers[l]
            h = torch.relu((2.0 * z[:, ia] - 1.0) @ W1.t() + b1)
            h = torch.relu(h @ W2.t() + b2)
            h = h @ W3.t() + b3
            y, ld = torch_pq(z[:, ib].clamp(0.0, 1.0), h.reshape(-1, len(ib), 2 * f.K + 1), f.K)
            z = z.index_copy(1, ib, y)
            out = out + ld
        return out

    ref_lq = fp64_logq(params64)
    assert float((lq.detach().double() - ref_lq.detach()).abs().max()) < 2e-3
    (ref_lq * c.double()).sum().backward()
    for a, p in zip(got, params64):
        scale = float(p.grad.abs().max())
        assert scale > 0
        assert float((a.double() - p.grad).abs().max()) < 2e-3 * scale
    for p, v in zip(f.parameters(), saved):
        assert torch.equal(p.detach(), v)


def test_native_sampling_is_its_density(cuda):
    """Points sampled by the hand-written inverse layer kernels carry the
    log density the density-direction kernels give them back, and the
    sampler is normalised (E_q[1/q] = 1)."""
    import torch

    f = _random_flow(18, 16, 3)
    assert not f.fused  # 9 x 33 outputs: beyond the tensor-core layer, the native sampler runs
    x, logq = f.sample(200_000, seed=9)
    lp = f.native_log_prob(x.float())
    assert float((lp.double() - logq).abs().max()) < 2e-3
    assert abs(torch.exp(-logq).mean().item() - 1.0) < 0.03
