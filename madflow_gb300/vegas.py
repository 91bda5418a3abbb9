"""VEGAS integration on the GPU with the interface madflow uses from
vegasflow (scripts/madflow_exec.py:487-525, utilities.py:90), and the
integrand contract f(x, n_dim, weight) (madflow_exec.py:422-470).

vegasflow itself is not part of the reference source; the integrator follows
Lepage's published algorithm (J. Comput. Phys. 27 (1978) 192): a separable
grid of ``nbins`` bins per dimension, per-iteration estimates combined with
inverse-variance weights, and the damped grid refinement (alpha = 1.5).
Uniform numbers come from Philox4x32-10 keyed by (seed, stream, iteration,
event), so a run is reproducible and the CPU oracle can replay it.

Two paths:
  * any Python callable integrand: uniforms, grid map and accumulation run in
    CUDA kernels, the integrand is called on (N, ndim) device tensors;
  * a ``FusedIntegrand`` (a madflow_gb300 process + configuration): one fused
    kernel per iteration (uniforms -> map -> phase space -> cuts -> PDF ->
    |M|^2 -> sums), optionally captured once as a CUDA graph and replayed.
"""
import ctypes
import math
import time
import warnings

import torch

from . import _lib
from .config import DTYPE, device, stream_ptr, to_device
from .matrix import PROCESSES

BINS_MAX = 50
ALPHA = 1.5


def _limit(events_limit):
    """events_limit for the C configuration: 0 = one slice."""
    if events_limit is None:
        return 0
    if int(events_limit) <= 0:
        raise ValueError(f"events_limit must be positive, not {events_limit}")
    return int(events_limit)


def _cut_table(cuts):
    """(variable, particle, min_val, max_val) tuples, as
    PhaseSpaceGenerator.register_cut takes them (None: no bound)."""
    cuts = list(cuts or [])
    if len(cuts) > _lib.MF_MAX_CUTS:
        raise ValueError(f"at most {_lib.MF_MAX_CUTS} cuts")
    out = []
    for variable, particle, lo, hi in cuts:
        if variable not in _lib.CUT_VARIABLES:
            raise ValueError(f"{variable} is not implemented")
        if particle is None:
            raise ValueError("a cut of the fused integrand names its particle")
        out.append((variable, int(particle), lo, hi))
    return out


def _cfg_struct(cfg):
    s = _lib.IntegrandConfig()
    for k, _ in _lib.IntegrandConfig._fields_:
        if k == "ncuts":
            s.ncuts = len(cfg["cuts"])
        elif k == "cuts":
            for i, (variable, particle, lo, hi) in enumerate(cfg["cuts"]):
                c = s.cuts[i]
                c.variable, c.particle = _lib.CUT_VARIABLES[variable], particle
                c.has_min, c.has_max = int(lo is not None), int(hi is not None)
                c.min_val = 0.0 if lo is None else float(lo)
                c.max_val = 0.0 if hi is None else float(hi)
        else:
            setattr(s, k, cfg[k])
    return s


class FusedIntegrand:
    """The integrand of one g g > t t~ + gluons process as a GPU kernel.

    kind 0: fixed partonic sqrt(s) (g g > t t~ only): rambo over 8 uniforms,
            f = |M|^2 * rambo weight * 389379365.6 / (2 s) pb.
    kind 1: hadronic sqrt(S): ramboflow over 4(n-2)+2 uniforms, synthetic gluon
            PDF at Q^2 = q2, cuts on the outgoing gluons,
            f = |M|^2 * lum * weight (madflow_exec.py:436-458).
    initial_states "gg": the g g process alone; "pp" (kind 1, n_gluons = 2):
            p p > t t~ at leading order, the g g channel plus the light-quark
            channels q q~ and q~ q (q = d u s c) with the synthetic quark
            densities, summed per event as madflow sums its processes.
    q2: the fixed scale Q^2 (default mt^2), or "dynamic": madflow's default
            scale, per event mu = sum of the outgoing m_T / 2, with alpha_s
            (then alpha_s(M_Z^2)) run to mu at one loop (mf_integrand_config).
    pt_cut: madflow's --pt_cut, p_T > pt_cut for every outgoing particle
            (tops included; kind 1), beside the gluon cuts ptmin, etamax,
            drmin.
    cuts:   up to 8 (variable, particle, min_val, max_val) as
            PhaseSpaceGenerator.register_cut takes them (pt, mt, mt2, eta;
            None for no bound), e.g. PhaseSpaceGenerator.cut_table(); kind 1.
    events_limit: run calls in slices of at most this many events (the
            handle's scratch holds one slice; the batch Newton rule runs per
            slice, as madflow's integrand sees one vegasflow slice per call);
            None: one slice.  VegasFlow(events_limit=...) overrides it for
            its iterations.
    """

    def __init__(self, n_gluons, kind=1, sqrts=13000.0, mt=173.0, wt=1.4915000200271606, alpha_s=0.118, ptmin=0.0,
                 etamax=0.0, drmin=0.0, q2=None, newton_rule=_lib.MF_NEWTON_BATCH, precision=None,
                 initial_states="gg", events_limit=None, pt_cut=None, cuts=None):
        if initial_states not in ("gg", "pp"):
            raise ValueError(f"initial_states must be 'gg' or 'pp', not {initial_states!r}")
        self.matrix = PROCESSES[n_gluons](precision=precision)
        self.initial_states = initial_states
        self.cfg = dict(kind=kind, sqrts=float(sqrts), mt=float(mt), wt=float(wt), alpha_s=float(alpha_s),
                        ptmin=float(ptmin), etamax=float(etamax), drmin=float(drmin),
                        q2=float(mt * mt if q2 is None else (-1.0 if q2 == "dynamic" else q2)),
                        newton_rule=int(newton_rule),
                        initial_states=_lib.MF_INITIAL_PP if initial_states == "pp" else _lib.MF_INITIAL_GG,
                        events_limit=_limit(events_limit), ptmin_all=float(pt_cut or 0.0),
                        cuts=_cut_table(cuts))
        self._cs = _cfg_struct(self.cfg)
        nd = ctypes.c_int()
        _lib.call("mf_integrand_ndim", self.matrix.handle, ctypes.byref(self._cs), ctypes.byref(nd))
        self.n_dim = nd.value

    def __call__(self, xrand, n_dim=None, weight=None, out=None):
        """f(x) for x (N, ndim); events failing the cuts give 0.

        x in page-locked host memory (a pinned float64 CPU tensor) is read
        by the kernels directly (mf_integrand_rows, zero-copy over the host
        link), as is `out` (optional, float64 (N,), pinned CPU or CUDA),
        which then receives f; other inputs are copied to the device first.
        Returns f (out if given)."""
        if isinstance(xrand, torch.Tensor) and xrand.device.type == "cpu" and xrand.is_pinned() \
                and xrand.dtype == DTYPE and xrand.dim() == 2 and xrand.is_contiguous():
            x = xrand
        else:
            x = to_device(xrand)
        if x.dim() != 2 or x.shape[1] != self.n_dim:
            raise ValueError(f"x must have shape (N, {self.n_dim}), got {tuple(x.shape)}")
        N = x.shape[0]
        if out is None:
            f = torch.empty(N, dtype=DTYPE, device=device())
        else:
            ok = out.dtype == DTYPE and out.dim() == 1 and out.shape[0] == N and out.is_contiguous() and (
                out.device.type == "cuda" or out.is_pinned())
            if not ok:
                raise ValueError("out must be a contiguous float64 (N,) CUDA or pinned CPU tensor")
            f = out
        _lib.call("mf_integrand_rows", self.matrix.handle, ctypes.byref(self._cs), x.data_ptr(), N, f.data_ptr(),
                  stream_ptr())
        return f

    def iteration(self, grid, seed, stream_id, iteration_dev, n_events, results, f_out=None, u_out=None,
                  events_limit=None):
        """One fused VEGAS iteration (mf_vegas_iteration); events_limit (if
        given) replaces the integrand's own for this call."""
        cs = self._cs
        if events_limit is not None:
            cs = _cfg_struct(dict(self.cfg, events_limit=_limit(events_limit)))
        _lib.call("mf_vegas_iteration", self.matrix.handle, ctypes.byref(cs), grid.data_ptr(),
                  grid.shape[1] - 1, int(seed), int(stream_id), iteration_dev.data_ptr(), int(n_events),
                  results.data_ptr(), f_out.data_ptr() if f_out is not None else None,
                  u_out.data_ptr() if u_out is not None else None, stream_ptr())

    def check_errors(self, clear=True):
        """Read the handle's device error state (synchronous).  Raises
        DeviceError when a bounded tensor-core wait ran out (bit 0 of
        mf_process_error_flags: the affected events got NaN); returns the
        number of non-finite event weights that entered the sums as 0 since
        the last check (mf_process_nonfinite)."""
        flags = ctypes.c_int()
        _lib.call("mf_process_error_flags", self.matrix.handle, ctypes.byref(flags), int(bool(clear)))
        count = ctypes.c_int64()
        st = _lib.load().mf_process_nonfinite(self.matrix.handle, ctypes.byref(count), int(bool(clear)))
        if st not in (_lib.MF_OK, _lib.MF_ERR_NONFINITE):
            raise _lib.MadflowError(st, "mf_process_nonfinite")
        if flags.value & 1:
            raise _lib.DeviceError("a bounded wait on the tensor cores ran out in the matrix-element kernel; "
                                   "the affected events were set to NaN")
        return int(count.value)

    def scratch_bytes(self):
        """Device bytes of scratch the handle holds (mf_process_scratch_bytes)."""
        b = ctypes.c_int64()
        _lib.call("mf_process_scratch_bytes", self.matrix.handle, ctypes.byref(b))
        return int(b.value)

    def set_wait_limit(self, tries):
        """Tries (~1 ms each) of each bounded tensor-core wait (default 1000)."""
        _lib.call("mf_process_set_wait_limit", self.matrix.handle, int(tries))

    def tuning(self):
        """The matrix-element launch configuration of the handle: colour sum
        on the SIMT lanes (0) or tensor cores (1), grid waves, whether the
        autotuner chose it, and the autotuner's time per variant in ms
        (index colour*4 + log2(waves); -1 where a variant does not exist)."""
        return self.matrix.tuning()

    def set_timing(self, enable=True):
        """Record CUDA events between the pipeline stages of later calls."""
        _lib.call("mf_process_set_timing", self.matrix.handle, int(bool(enable)))

    def stage_ms(self):
        """Milliseconds of the last call's stages (phase-space first pass with
        the batch Newton minimum, phase space, matrix element, accumulation);
        the caller synchronises first."""
        ms = (ctypes.c_float * _lib.MF_STAGES)()
        _lib.call("mf_process_stage_ms", self.matrix.handle, ms)
        return dict(zip(("seed", "phase_space", "matrix_element", "accumulate"), list(ms)))


def reduce_results(results, group=None):
    """Sum an iteration's results vector [2 + ndim*nbins] (sum of w, of w^2,
    per-bin w^2) over the ranks of a torch.distributed group, in place: the
    one exchange of a sharded integration.  The vector stays on its device
    for NCCL and goes through host memory for gloo."""
    import torch.distributed as dist

    if group is None and not dist.is_initialized():
        return results
    if dist.get_backend(group) == "nccl" or results.device.type == "cpu":
        dist.all_reduce(results, op=dist.ReduceOp.SUM, group=group)
        return results
    host = results.cpu()
    dist.all_reduce(host, op=dist.ReduceOp.SUM, group=group)
    results.copy_(host)
    return results


def iteration_estimate(s1, s2, n_per_rank, world=1):
    """(estimate, sigma) of one iteration from the summed w = f jac / n and
    w^2 over world ranks of n events each: the mean of f jac over all
    M = world*n events and the error of that mean."""
    n, m = float(n_per_rank), float(n_per_rank) * world
    if world == 1:
        # the unsharded expression (VegasFlow.run_event), so one rank gives
        # the same bits
        var = (n * s2 - s1 * s1) / (n - 1.0)
        return s1, math.sqrt(max(var, 0.0))
    res = s1 / world
    var = n * n * (s2 - s1 * s1 / m) / (m * (m - 1.0))
    return res, math.sqrt(max(var, 0.0))


class VegasFlow:
    """VEGAS integrator (the vegasflow interface madflow calls).

    >>> vegas = VegasFlow(n_dim, n_events)
    >>> vegas.compile(integrand)
    >>> res, err = vegas.run_integration(n_iter)
    """

    def __init__(self, n_dim, n_events, events_limit=None, seed=4, nbins=BINS_MAX, alpha=ALPHA, stream_id=0,
                 verbose=False, use_graph=True, process_group=None):
        """process_group (torch.distributed, optional): shard every iteration
        over the group's ranks, n_events on each (Philox stream
        stream_id * world + rank), with one all-reduce of the results vector
        per iteration; every rank then refines the same grid."""
        self.n_dim = int(n_dim)
        self.n_events = int(n_events)
        self.events_per_run = int(events_limit or n_events)
        self.seed = int(seed)
        self.group = process_group
        self.world, self.rank = 1, 0
        if process_group is not None:
            import torch.distributed as dist

            self.world, self.rank = dist.get_world_size(process_group), dist.get_rank(process_group)
        self.stream_id = int(stream_id) * self.world + self.rank
        self.nbins = int(nbins)
        self.alpha = float(alpha)
        self.verbose = verbose
        self.use_graph = use_graph
        self.train = True
        self.grid = torch.linspace(0.0, 1.0, self.nbins + 1, dtype=DTYPE, device=device()).repeat(self.n_dim, 1)
        self.grid = self.grid.contiguous()
        self.iteration = torch.zeros(1, dtype=torch.int32, device=device())
        self.width = 2 + self.n_dim * self.nbins
        self.results = torch.zeros(self.width, dtype=DTYPE, device=device())
        self.history = []  # (result, sigma) per iteration
        self.nonfinite = 0  # event weights that were not finite and entered the sums as 0
        self.integrand = None
        self._graph = None

    # --- vegasflow API -------------------------------------------------------
    def compile(self, integrand, compilable=True):
        self.integrand = integrand
        self._graph = None
        if isinstance(integrand, FusedIntegrand) and integrand.n_dim != self.n_dim:
            raise ValueError(f"integrand has {integrand.n_dim} dimensions, the integrator {self.n_dim}")

    def freeze_grid(self):
        self.train = False
        self._graph = None

    def unfreeze_grid(self):
        self.train = True
        self._graph = None

    def set_seed(self, seed):
        self.seed = int(seed)
        self._graph = None

    # --- one iteration ---------------------------------------------------------
    def _iteration_python(self):
        res = self.results
        res.zero_()
        tmp = torch.empty_like(res)
        done = 0
        it = int(self.iteration.item())
        while done < self.n_events:
            n = min(self.events_per_run, self.n_events - done)
            u = torch.empty((self.n_dim, n), dtype=DTYPE, device=device())
            _lib.call("mf_philox_uniforms", self.seed, self.stream_id, it, done, n, self.n_dim, u.data_ptr(),
                      stream_ptr())
            x = torch.empty_like(u)
            jac = torch.empty(n, dtype=DTYPE, device=device())
            bins = torch.empty((self.n_dim, n), dtype=torch.int32, device=device())
            _lib.call("mf_vegas_sample", self.grid.data_ptr(), self.n_dim, self.nbins, u.data_ptr(), n, x.data_ptr(),
                      jac.data_ptr(), bins.data_ptr(), stream_ptr())
            f = self.integrand(x.T, n_dim=self.n_dim, weight=jac / self.n_events)
            f = to_device(f).reshape(-1)
            bad = ~torch.isfinite(f)
            nbad = int(bad.sum())
            if nbad:
                # counted and zeroed, as the fused path does on the device
                f = torch.where(bad, torch.zeros_like(f), f)
                self._note_nonfinite(nbad)
            _lib.call("mf_vegas_accumulate", f.data_ptr(), jac.data_ptr(), bins.data_ptr(), n, self.n_dim,
                      self.nbins, 1.0 / self.n_events, tmp.data_ptr(), stream_ptr())
            res += tmp
            done += n
        if self.train:
            _lib.call("mf_vegas_refine", self.grid.data_ptr(), res[2:].data_ptr(), self.n_dim, self.nbins, self.alpha,
                      stream_ptr())
        self.iteration += 1

    def _refine(self):
        _lib.call("mf_vegas_refine", self.grid.data_ptr(), self.results[2:].data_ptr(), self.n_dim, self.nbins,
                  self.alpha, stream_ptr())

    def _fused_limit(self):
        return self.events_per_run if self.events_per_run < self.n_events else None

    def _iteration_fused_body(self):
        self.integrand.iteration(self.grid, self.seed, self.stream_id, self.iteration, self.n_events, self.results,
                                 events_limit=self._fused_limit())
        if self.train:
            self._refine()
        self.iteration += 1

    def _iteration_sharded(self):
        if isinstance(self.integrand, FusedIntegrand):
            self.integrand.iteration(self.grid, self.seed, self.stream_id, self.iteration, self.n_events, self.results,
                                     events_limit=self._fused_limit())
        else:
            train, self.train = self.train, False
            self._iteration_python()
            self.train = train
            self.iteration -= 1
        reduce_results(self.results, self.group)
        if self.train:
            self._refine()
        self.iteration += 1

    def _iteration_fused(self):
        if not self.use_graph:
            self._iteration_fused_body()
            return
        if self._graph is None:
            # one uncaptured iteration allocates the scratch and uploads tables
            self._iteration_fused_body()
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self._iteration_fused_body()
            torch.cuda.current_stream().wait_stream(s)
            self._graph = g
            # capturing recorded but did not run the body: the warm-up above was iteration it
            return
        self._graph.replay()

    def _note_nonfinite(self, n):
        self.nonfinite += n
        warnings.warn(f"{n} non-finite event weights entered iteration {len(self.history) + 1} as 0",
                      RuntimeWarning, stacklevel=3)

    def _check_device(self):
        """After an iteration's results reached the host: raise if a kernel
        reported a tensor-core timeout, count zeroed non-finite weights."""
        if isinstance(self.integrand, FusedIntegrand):
            n = self.integrand.check_errors()
            if n:
                self._note_nonfinite(n)

    def run_event(self):
        if self.group is not None:
            self._iteration_sharded()
            r = self.results[:2].double().cpu().numpy()
            self._check_device()
            return iteration_estimate(float(r[0]), float(r[1]), self.n_events, self.world)
        if isinstance(self.integrand, FusedIntegrand):
            self._iteration_fused()
        else:
            self._iteration_python()
        r = self.results[:2].double().cpu().numpy()
        self._check_device()
        n = self.n_events
        res = float(r[0])
        var = (n * float(r[1]) - res * res) / (n - 1.0)
        return res, math.sqrt(max(var, 0.0))

    def run_integration(self, n_iter, log_time=True, target_rel_error=None):
        """Run ``n_iter`` iterations; returns the inverse-variance weighted
        (result, error) over the iterations of this call.  With
        ``target_rel_error`` it stops as soon as the combined error reaches it."""
        if self.integrand is None:
            raise RuntimeError("compile() an integrand first")
        wsum = wres = 0.0
        self.last_run = []
        for _ in range(int(n_iter)):
            t0 = time.perf_counter()
            res, sig = self.run_event()
            dt = time.perf_counter() - t0
            self.history.append((res, sig))
            self.last_run.append((res, sig, dt))
            if sig > 0:
                w = 1.0 / (sig * sig)
                wsum += w
                wres += w * res
            if self.verbose:
                print(f"iteration {len(self.history)}: {res:.6g} +/- {sig:.3g} ({dt:.3f}s)")
            if target_rel_error is not None and wsum > 0:
                cur = wres / wsum
                if cur != 0 and (1.0 / math.sqrt(wsum)) / abs(cur) <= target_rel_error:
                    break
        if wsum == 0:
            return (self.history[-1][0] if self.history else 0.0), 0.0
        return wres / wsum, 1.0 / math.sqrt(wsum)


def vegas_wrapper(integrand, n_dim, n_iter, total_n_events, compilable=True, seed=4, **kw):
    """vegasflow.vegas_wrapper: compile, run ``n_iter`` iterations, return (res, err)."""
    v = VegasFlow(n_dim, total_n_events, seed=seed, **kw)
    v.compile(integrand, compilable)
    return v.run_integration(n_iter)
