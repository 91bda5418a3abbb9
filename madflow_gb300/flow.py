"""Normalizing-flow importance sampler over the unit hypercube, an alternative
proposal to the VEGAS grid (no counterpart in the reference).

Architecture (Mueller et al., "Neural Importance Sampling", ACM TOG 38 (2019)
145): ``n_layers`` piecewise-quadratic coupling layers; each transforms half
of the dimensions with bins (K widths, K+1 vertex heights) predicted by an MLP
of ``n_hidden`` hidden layers of ``hidden`` units from the other half.

Compute split (two hidden layers of 64 units, 4, 8 or 16 bins, at most 16
dimensions per half):
  * training runs in hand-written FP32 kernels (``mf_flow_train.cu``): per
    coupling layer, the MLP and the transform in the density direction, and
    their gradient (the MLP backward as tiled GEMMs in shared memory, the
    transform's backward per point and dimension, weight gradients summed in
    a fixed order); Adam updates the weights;
  * sampling runs one tcgen05 kernel per coupling layer (``mf_flow_tc.cu``:
    the MLP as three GEMMs on TF32 or BF16 operands with FP32 tensor-memory
    accumulators, the inverse transform in the epilogue) when the layer fits
    it (its MLP outputs in at most two chunks of whole dimensions, 256
    columns each) and TF32 (``tf32=True``) or BF16 (``tc_bf16=True``) is
    chosen, else the hand-written FP32 layer kernel.
Other shapes, and ``bf16=True``, run the conditioner through torch (cuBLAS,
BF16 under autocast) with the hand-written transform kernels of
``mf_flow.cu`` (forward, inverse, log-Jacobian, backward).

Training minimises the variance of the weights f/q with the score-function
gradient  d Var/d theta = -E_q[(f/q)^2 d log q/d theta]  on batches drawn from
the flow itself; the integral estimate mean(f/q) stays unbiased for any
trained state, and each integration iteration uses one frozen state.
"""
import ctypes
import math
import time

import torch

from . import _lib
from .config import device, stream_ptr


class _PQ(torch.autograd.Function):
    """y = CDF(x), logdet = sum log pdf(x) for one coupling layer (CUDA)."""

    @staticmethod
    def forward(ctx, x_b, params, K):
        x_b = x_b.contiguous()
        params = params.contiguous()
        n, nb = x_b.shape
        y = torch.empty_like(x_b)
        ld = torch.empty(n, dtype=torch.float32, device=x_b.device)
        _lib.call("mf_pq_forward", x_b.data_ptr(), params.data_ptr(), n, nb, K, y.data_ptr(), ld.data_ptr(),
                  stream_ptr())
        ctx.save_for_backward(x_b, params)
        ctx.K = K
        return y, ld

    @staticmethod
    def backward(ctx, gy, gld):
        x_b, params = ctx.saved_tensors
        n, nb = x_b.shape
        gy = gy.contiguous() if gy is not None else None
        gld = gld.contiguous() if gld is not None else None
        gx = torch.empty_like(x_b)
        gp = torch.empty_like(params)
        _lib.call("mf_pq_backward", x_b.data_ptr(), params.data_ptr(), gy.data_ptr() if gy is not None else None,
                  gld.data_ptr() if gld is not None else None, n, nb, ctx.K, gx.data_ptr(), gp.data_ptr(),
                  stream_ptr())
        return gx, gp, None


def pq_forward(x_b, params, K):
    return _PQ.apply(x_b, params, K)


def pq_inverse(u_b, params, K):
    u_b = u_b.contiguous()
    params = params.contiguous()
    n, nb = u_b.shape
    x = torch.empty_like(u_b)
    ld = torch.empty(n, dtype=torch.float32, device=u_b.device)
    _lib.call("mf_pq_inverse", u_b.data_ptr(), params.data_ptr(), n, nb, K, x.data_ptr(), ld.data_ptr(), stream_ptr())
    return x, ld


def _masks(dim, n_layers, seed):
    """Balanced random partitions; layers 2j and 2j+1 are complementary so
    every dimension is transformed n_layers/2 times."""
    g = torch.Generator().manual_seed(seed)
    masks = []
    for j in range((n_layers + 1) // 2):
        perm = torch.randperm(dim, generator=g)
        m = torch.zeros(dim, dtype=torch.bool)
        m[perm[: dim // 2]] = True
        masks += [m, ~m]
    return masks[:n_layers]


def _tc_chunks_fit(nb, np_):
    """Whether nb dimensions of np_ parameters fit the tensor-core sampling
    layer's third GEMM: at most 256 columns in its first chunk of whole
    dimensions, the rest (padded to 16) at most 256 in a second."""
    da = min(nb, 256 // np_)
    return ((nb - da) * np_ + 15) // 16 * 16 <= 256


class NormalizingFlow(torch.nn.Module):
    def __init__(self, dim, n_layers=6, bins=16, hidden=64, n_hidden=2, seed=0, bf16=False, tf32=False, fused=None,
                 native=None, tc_bf16=False):
        """native: train (and sample, where the tensor-core layer does not
        apply) with the hand-written FP32 layer kernels; by default whenever
        the shapes fit them (64 hidden units, two hidden layers, 4, 8 or 16
        bins, at most 16 dimensions per half, nb (2K+1) <= 320) and bf16 is
        not set.  bf16: conditioner GEMMs in BF16 through torch autocast
        (cuBLAS) instead.  fused: sample with one tensor-core kernel per
        coupling layer (mf_flow_inv_layer_tc: the MLP in TF32 and the inverse
        transform); by default whenever tf32 is set and the shapes fit it
        (also the MLP outputs in at most two chunks of whole dimensions, 256
        columns each).  tc_bf16: the fused sampling kernel with BF16 GEMM
        operands (mf_flow_inv_layer_tc_bf16) instead of TF32; it implies
        fused sampling, and training stays in the FP32 layer kernels.
        Reduced-precision GEMMs leave the estimates
        unbiased (the sampled log-density is the exact density of the map as
        evaluated); they perturb the training gradients."""
        super().__init__()
        if tc_bf16 and bf16:
            raise ValueError("tc_bf16 (hand-written BF16 sampling) and bf16 (torch autocast) exclude each other")
        self.dim, self.K, self.bf16, self.tf32, self.tc_bf16 = dim, bins, bf16, tf32, bool(tc_bf16)
        self.masks = _masks(dim, n_layers, seed)
        self.nets = torch.nn.ModuleList()
        torch.manual_seed(seed)
        for m in self.masks:
            nb, na = int(m.sum()), int((~m).sum())
            layers = [torch.nn.Linear(na, hidden), torch.nn.ReLU()]
            for _ in range(n_hidden - 1):
                layers += [torch.nn.Linear(hidden, hidden), torch.nn.ReLU()]
            last = torch.nn.Linear(hidden, nb * (2 * bins + 1))
            torch.nn.init.zeros_(last.weight)  # start at the identity map
            torch.nn.init.zeros_(last.bias)
            layers.append(last)
            self.nets.append(torch.nn.Sequential(*layers))
        self.to(device())
        self._idx = [(torch.nonzero(m).flatten().to(device()), torch.nonzero(~m).flatten().to(device()))
                     for m in self.masks]
        self._idx32 = [(ib.int().contiguous(), ia.int().contiguous()) for ib, ia in self._idx]
        fits = (hidden == 64 and n_hidden == 2 and bins in (4, 8, 16)
                and all(0 < len(ia) <= 16 and 0 < len(ib) <= 16 and _tc_chunks_fit(len(ib), 2 * bins + 1)
                        for ib, ia in self._idx))
        if (fused or tc_bf16) and not fits:
            raise ValueError("the fused sampling kernel needs 64 hidden units, 2 hidden layers, 4/8/16 bins, "
                             "at most 16 dimensions per half and two chunks of at most 256 MLP outputs")
        self.fused = bool(fits and ((tf32 or tc_bf16) and not bf16) if fused is None else fused)
        if self.tc_bf16 and not self.fused:
            raise ValueError("tc_bf16 samples with the fused kernel")
        nfits = (hidden == 64 and n_hidden == 2 and bins in (4, 8, 16)
                 and all(0 < len(ia) <= 16 and 0 < len(ib) <= 16 and len(ib) * (2 * bins + 1) <= 320
                         for ib, ia in self._idx))
        if native and not nfits:
            raise ValueError("the native layer kernels need 64 hidden units, 2 hidden layers, 4/8/16 bins, "
                             "at most 16 dimensions per half and nb (2K+1) <= 320")
        self.native = bool(nfits and not bf16 if native is None else native)
        if self.native:
            ws = 0
            for ib, ia in self._idx:
                b = ctypes.c_int64()
                _lib.call("mf_flow_layer_grad_workspace", len(ia), len(ib), bins, ctypes.byref(b))
                ws = max(ws, b.value)
            self._workspace = torch.empty(ws // 4 + 1, dtype=torch.float32, device=device())
            for p in self.parameters():
                p.grad = torch.zeros_like(p)

    def _layer_ptrs(self, l):
        """Device pointers of layer l's weights (W1, b1, W2, b2, W3, b3)."""
        net = self.nets[l]
        return [t.data_ptr() for t in (net[0].weight, net[0].bias, net[2].weight, net[2].bias, net[4].weight,
                                       net[4].bias)]

    def _layer_grad_ptrs(self, l):
        net = self.nets[l]
        ts = (net[0].weight, net[0].bias, net[2].weight, net[2].bias, net[4].weight, net[4].bias)
        for t in ts:
            if t.grad is None:  # after zero_grad(set_to_none=True)
                t.grad = torch.zeros_like(t)
        return [t.grad.data_ptr() for t in ts]

    @torch.no_grad()
    def native_backward(self, x, glogq):
        """Gradient of L = sum_i glogq_i log q(x_i) with respect to every
        weight, in the hand-written kernels: the density direction through
        all layers (storing each layer's input), then the layers' gradients
        in reverse.  Writes p.grad of every parameter (overwriting) and
        returns log q(x) (float32)."""
        n = x.shape[0]
        z = x.float().contiguous()
        logq = torch.zeros(n, dtype=torch.float32, device=z.device)
        gl = glogq.float().contiguous()
        inputs = []
        for l in reversed(range(len(self.masks))):
            ib, ia = self._idx32[l]
            zn = torch.empty_like(z)
            _lib.call("mf_flow_layer_density", z.data_ptr(), zn.data_ptr(), n, self.dim, ia.data_ptr(), len(ia),
                      ib.data_ptr(), len(ib), self.K, *self._layer_ptrs(l), logq.data_ptr(), stream_ptr())
            inputs.append(z)
            z = zn
        g = torch.zeros_like(z)
        for j, l in enumerate(range(len(self.masks))):
            ib, ia = self._idx32[l]
            zin = inputs[len(inputs) - 1 - j]
            gin = torch.empty_like(zin)
            _lib.call("mf_flow_layer_grad", zin.data_ptr(), g.data_ptr(), gin.data_ptr(), n, self.dim, ia.data_ptr(),
                      len(ia), ib.data_ptr(), len(ib), self.K, *self._layer_ptrs(l), gl.data_ptr(),
                      *self._layer_grad_ptrs(l), self._workspace.data_ptr(), self._workspace.numel() * 4,
                      stream_ptr())
            g = gin
        return logq

    @torch.no_grad()
    def native_log_prob(self, x):
        """log q(x) through the hand-written density-direction kernels."""
        n = x.shape[0]
        z = x.float().contiguous().clone()
        logq = torch.zeros(n, dtype=torch.float32, device=z.device)
        for l in reversed(range(len(self.masks))):
            ib, ia = self._idx32[l]
            _lib.call("mf_flow_layer_density", z.data_ptr(), z.data_ptr(), n, self.dim, ia.data_ptr(), len(ia),
                      ib.data_ptr(), len(ib), self.K, *self._layer_ptrs(l), logq.data_ptr(), stream_ptr())
        return logq

    def _params(self, l, x_a):
        if self.bf16:
            with torch.autocast("cuda", dtype=torch.bfloat16):
                out = self.nets[l](2.0 * x_a - 1.0)
        else:
            # FP32 weights and activations; TF32 tensor-core GEMMs if asked
            prev = torch.backends.cuda.matmul.allow_tf32
            torch.backends.cuda.matmul.allow_tf32 = bool(self.tf32)
            try:
                out = self.nets[l](2.0 * x_a - 1.0)
            finally:
                torch.backends.cuda.matmul.allow_tf32 = prev
        nb = int(self.masks[l].sum())
        return out.float().reshape(-1, nb, 2 * self.K + 1)

    @torch.no_grad()
    def sample(self, n, seed=1234, iteration=0, stream_id=7):
        """n points (float64 (n, dim)) and their log density (float64 (n,))."""
        u = torch.empty((self.dim, n), dtype=torch.float64, device=device())
        _lib.call("mf_philox_uniforms", int(seed), int(stream_id), int(iteration), 0, n, self.dim, u.data_ptr(),
                  stream_ptr())
        z = u.T.float().contiguous()
        logq = torch.zeros(n, dtype=torch.float32, device=device())
        if self.fused:
            fn = "mf_flow_inv_layer_tc_bf16" if self.tc_bf16 else "mf_flow_inv_layer_tc"
            err = torch.zeros(1, dtype=torch.int32, device=device())
            for l, net in enumerate(self.nets):
                ib, ia = self._idx32[l]
                w = [t.detach().float().contiguous() for t in (net[0].weight, net[0].bias, net[2].weight,
                                                               net[2].bias, net[4].weight, net[4].bias)]
                _lib.call(fn, z.data_ptr(), n, self.dim, ia.data_ptr(), len(ia), ib.data_ptr(), len(ib), self.K,
                          *[t.data_ptr() for t in w], logq.data_ptr(), err.data_ptr(), stream_ptr())
            if int(err.item()) != 0:
                raise RuntimeError(f"{fn}: device error flag {int(err.item())}")
            return z.double(), logq.double()
        if self.native:
            for l in range(len(self.masks)):
                ib, ia = self._idx32[l]
                _lib.call("mf_flow_layer_sample", z.data_ptr(), z.data_ptr(), n, self.dim, ia.data_ptr(), len(ia),
                          ib.data_ptr(), len(ib), self.K, *self._layer_ptrs(l), logq.data_ptr(), stream_ptr())
            return z.double(), logq.double()
        for l in range(len(self.masks)):
            ib, ia = self._idx[l]
            params = self._params(l, z[:, ia])
            xb, ld = pq_inverse(z[:, ib], params, self.K)
            z[:, ib] = xb
            logq += ld
        return z.double(), logq.double()

    def log_prob(self, x):
        """log q(x) with gradients w.r.t. the network weights."""
        z = x.float()
        logq = torch.zeros(x.shape[0], dtype=torch.float32, device=x.device)
        for l in reversed(range(len(self.masks))):
            ib, ia = self._idx[l]
            params = self._params(l, z[:, ia])
            yb, ld = pq_forward(z[:, ib], params, self.K)
            z = z.index_copy(1, ib, yb)
            logq = logq + ld
        return logq


def _clamp_open(x, eps=1e-7):
    return x.clamp(eps, 1.0 - eps)


def _backward(flow, loss):
    """loss.backward() with the conditioner's GEMMs in the flow's precision
    (TF32 tensor cores when the flow runs its forward GEMMs in TF32)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = bool(getattr(flow, "tf32", False)) or prev
    try:
        loss.backward()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


class _GraphedStep:
    """One Adam step on the mean log-density of a fixed number of points,
    captured once as a CUDA graph (the log-density, its backward pass with
    the custom coupling kernels and the optimizer step: some hundred small
    launches, replayed as one).  The optimizer must be capturable.  The
    warm-up steps the capture needs run on a placeholder batch; the weights
    and the optimizer state are put back afterwards."""

    def __init__(self, flow, opt, n):
        self.flow, self.opt = flow, opt
        self.x = torch.full((n, flow.dim), 0.5, dtype=torch.float32, device=device())
        self.gl = torch.full((n,), -1.0 / n, dtype=torch.float32, device=device())
        params = list(flow.parameters())
        saved = [p.detach().clone() for p in params]
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                self._step()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._step()
        with torch.no_grad():
            for p, v in zip(params, saved):
                p.copy_(v)
        for st in opt.state.values():
            for v in st.values():
                if torch.is_tensor(v):
                    v.zero_()

    def _step(self):
        if self.flow.native:
            # the loss -mean log q: dL/dlog q_i = -1/n; the kernels overwrite p.grad
            self.flow.native_backward(self.x, self.gl)
        else:
            self.opt.zero_grad(set_to_none=False)
            loss = -self.flow.log_prob(self.x).mean()
            _backward(self.flow, loss)
        self.opt.step()

    def __call__(self, xs):
        self.x.copy_(xs)
        self.graph.replay()


def _train_step(flow, opt, x, w, minibatch, resample=0, step=None, steps=1):
    """Variance-loss updates on one batch (x, w = f/q) drawn from the flow.

    The gradient of Var(f/q) is -E_q[w^2 d log q] (score function).  With
    resample > 0 it is estimated from `resample` events drawn with
    probability w^2 / sum w^2 (systematic resampling), as
    -(sum w^2) mean(d log q) over them: unbiased, and only the resampled
    events go through the flow's log-density and its backward pass.
    step (optional): a _GraphedStep for `resample` points (one minibatch).
    steps: optimiser steps on the batch, each on its own resample."""
    if resample > 0:
        w2 = (w * w).double()
        total = float(w2.sum())
        if total <= 0.0:
            return
        cdf = torch.cumsum(w2, 0) / total
        for _ in range(int(steps)):
            u = (torch.arange(resample, device=w.device, dtype=torch.float64)
                 + torch.rand(1, device=w.device, dtype=torch.float64)) / resample
            idx = torch.clamp(torch.searchsorted(cdf, u), max=w.numel() - 1)
            _resampled_step(flow, opt, x[idx], minibatch, resample, step)
        return
    mean_w = w.mean()
    scale = (mean_w * mean_w).clamp_min(1e-300)
    n = x.shape[0]
    for s in range(0, n, minibatch):
        wm = w[s: s + minibatch]
        coef = (wm * wm / scale).float()
        if flow.native:
            flow.native_backward(x[s: s + minibatch], -coef / wm.shape[0])
        else:
            lq = flow.log_prob(x[s: s + minibatch])
            loss = -(coef * lq).mean()
            opt.zero_grad(set_to_none=True)
            _backward(flow, loss)
        opt.step()


def _resampled_step(flow, opt, xs, minibatch, resample, step):
    """One optimiser step of -mean log q over resampled points xs."""
    if step is not None:
        step(xs)
        return
    for s in range(0, resample, minibatch):
        xm = xs[s: s + minibatch]
        if flow.native:
            flow.native_backward(xm, torch.full((xm.shape[0],), -1.0 / xm.shape[0], dtype=torch.float32,
                                                device=xm.device))
        else:
            loss = -flow.log_prob(xm).mean()
            opt.zero_grad(set_to_none=True)
            _backward(flow, loss)
        opt.step()


def train_flow(flow, integrand, n_batches=20, batch_size=1_000_000, minibatch=100_000, lr=2e-3, seed=99,
               log=None):
    """Variance-loss training on weights f/q of batches drawn from the flow."""
    opt = torch.optim.Adam(flow.parameters(), lr=lr)
    hist = []
    for b in range(n_batches):
        x, logq = flow.sample(batch_size, seed=seed, iteration=b)
        x = _clamp_open(x)
        w = integrand(x) * torch.exp(-logq)
        mean_w = float(w.mean())
        _train_step(flow, opt, x, w, minibatch)
        rel = float(w.std()) / mean_w if mean_w != 0 else float("nan")
        hist.append(rel)
        if log:
            log(f"flow batch {b}: mean {mean_w:.5g}, std/mean {rel:.4f}")
    return hist


def _vegas_map(grid, z):
    """x = G(z) through a frozen VEGAS grid [ndim][nb+1]; returns (x (N, ndim), jac)."""
    n, dim = z.shape
    u = z.T.contiguous()
    x = torch.empty_like(u)
    jac = torch.empty(n, dtype=torch.float64, device=z.device)
    bins = torch.empty((dim, n), dtype=torch.int32, device=z.device)
    _lib.call("mf_vegas_sample", grid.data_ptr(), dim, grid.shape[1] - 1, u.data_ptr(), n, x.data_ptr(),
              jac.data_ptr(), bins.data_ptr(), stream_ptr())
    return x.T, jac


def adaptive_flow_integration(flow, integrand, target_rel_error=1e-3, batch_size=1_000_000, max_batches=200,
                              train_batches=30, minibatch=100_000, lr=2e-3, seed=99, grid=None, prior=None,
                              resample=0, graph=True, train_steps=1):
    """Integrate while training: every batch is drawn from the current (frozen)
    flow, so mean(f/q) over it is an unbiased estimate with variance
    var(f/q)/n; the estimates of all batches are combined with
    inverse-variance weights (as VEGAS combines its iterations), and the first
    ``train_batches`` batches also update the flow afterwards.  Stops when the
    combined relative error reaches ``target_rel_error``.

    grid (optional): a frozen VEGAS grid [ndim][nb+1]; the flow then models
    the density of the grid's input variables, x = G(z), and the weights are
    f(G(z)) |dG/dz| / q(z).  prior (optional): (wsum, wres) of earlier
    unbiased estimates (e.g. the VEGAS iterations that adapted the grid), in
    the same inverse-variance form.  resample > 0: train on that many events
    resampled with probability w^2 (see _train_step).  graph: with
    resample > 0 and resample <= minibatch, the training step runs as a
    captured CUDA graph (_GraphedStep); train_steps optimiser steps per
    trained batch, each on its own resample.

    Returns (result, error, info)."""
    graphed = bool(graph and 0 < resample <= minibatch and train_batches > 0)
    opt = torch.optim.Adam(flow.parameters(), lr=lr, capturable=graphed)
    step = _GraphedStep(flow, opt, int(resample)) if graphed else None
    wsum, wres = prior if prior is not None else (0.0, 0.0)
    rel_std = float("nan")
    b = 0
    for b in range(int(max_batches)):
        z, logq = flow.sample(batch_size, seed=seed, iteration=b)
        z = _clamp_open(z)
        if grid is None:
            w = integrand(z) * torch.exp(-logq)
        else:
            x, jac = _vegas_map(grid, z)
            w = integrand(x) * jac * torch.exp(-logq)
        mv = torch.stack([w.mean(), w.var()]).tolist()
        res, var = mv[0], mv[1] / w.numel()
        rel_std = math.sqrt(max(mv[1], 0.0)) / res if res != 0 else float("nan")
        if var > 0:
            wsum += 1.0 / var
            wres += res / var
            cur = wres / wsum
            if cur != 0 and (1.0 / math.sqrt(wsum)) / abs(cur) <= target_rel_error:
                break
        if b < train_batches:
            _train_step(flow, opt, z, w, minibatch, resample, step, train_steps)
    info = {"batches": b + 1, "trained": min(b + 1, int(train_batches)), "last_rel_std": rel_std}
    if wsum == 0:
        return 0.0, 0.0, info
    return wres / wsum, 1.0 / math.sqrt(wsum), info


class FlowIntegrator:
    """Importance-sampling integration with a (frozen) flow proposal."""

    def __init__(self, flow, integrand, n_events, seed=4321):
        self.flow, self.integrand, self.n_events, self.seed = flow, integrand, int(n_events), seed
        self.history = []

    def run_event(self, it):
        x, logq = self.flow.sample(self.n_events, seed=self.seed, iteration=it)
        x = _clamp_open(x)
        w = self.integrand(x) * torch.exp(-logq)
        n = w.numel()
        res = float(w.mean())
        var = float(w.var()) / n
        self.last_eff = float(w.mean() / w.max()) if float(w.max()) > 0 else 0.0
        return res, math.sqrt(max(var, 0.0))

    def run_integration(self, n_iter, target_rel_error=None):
        wsum = wres = 0.0
        self.last_run = []
        for it in range(int(n_iter)):
            t0 = time.perf_counter()
            res, sig = self.run_event(len(self.history))
            self.history.append((res, sig))
            self.last_run.append((res, sig, time.perf_counter() - t0))
            if sig > 0:
                wsum += 1.0 / (sig * sig)
                wres += res / (sig * sig)
            if target_rel_error is not None and wsum > 0:
                cur = wres / wsum
                if cur != 0 and (1.0 / math.sqrt(wsum)) / abs(cur) <= target_rel_error:
                    break
        return (wres / wsum, 1.0 / math.sqrt(wsum)) if wsum > 0 else (0.0, 0.0)
