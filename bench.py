"""Benchmark: |M|^2 evaluations per second of the g g > t t~ + gluons
integrand inside fused VEGAS iterations on one GB300, the time to reach a
1e-3 relative integration error, and the error of the mixed-precision path.

    python bench.py [--config c1|c2|c3|c4|c5] [--gpus N] [--steps K] [--warmup W]
                    [--events N] [--impl reference]

A step is one fused VEGAS iteration over --events phase-space points (Philox
uniforms -> grid map -> phase space -> cuts -> PDF -> |M|^2 -> sums ->
refinement).  One JSON line is printed by rank 0.  The default workload is
c3, g g > t t~ g g at 13 TeV with the synthetic gluon PDF and the cuts
pT > 60 GeV, |eta| < 2.5, Delta R > 0.4, 10^7 points per iteration; the other
configurations are

  c1  g g > t t~ at fixed partonic sqrt(s) = 1 TeV, FP64, 5 x 10^6 points,
      integral checked against the oracle's replay of the same iterations
  c2  g g > t t~ g, pT > 30 GeV, |eta| < 4, 10 x 10^7 points, FP64 and mixed
  c4  the c3 integrand with the normalizing-flow proposal of the configuration
      (6 coupling layers, 16 bins, MLP 2 x 64, BF16 GEMMs, 20 training batches
      of 10^6) against plain VEGAS: time, events, unweighting efficiency
  c5  g g > t t~ g g g, c3 cuts, 10^6 points per iteration, mixed; flow
      against VEGAS on an equal event budget
  pp  p p > t t~ at leading order: g g > t t~ and the light-quark channels
      q q~ > t t~ (and mirror images) with synthetic quark densities, 10^7
      points per iteration, FP64 and mixed, and the quark channels' share

--gpus N without a torchrun environment starts N ranks itself (one per GPU,
weak scaling: every rank integrates its own Philox stream and the iteration
sums are all-reduced).  --impl reference times the reference's CPU path (the
oracle's C++/OpenMP restatement of madflow's integrand, timing build, all
host cores) on a bounded sample of the same workload.
"""
import argparse
import json
import math
import os
import platform
import socket
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s to 1e-3 rel. error & |M|^2 evals/s, gg>tt~gg, flow+mixed vs plain VEGAS, 1 GB300"
MT, WT, ALPHA_S = 173.0, 1.4915000200271606, 0.118
# Algorithmic flops per phase-space point of the colour-ordered evaluation
# (all helicities, no sharing across helicities; complex mul 6, add 2,
# div/sqrt/log 1), counted by the oracle's counting scalar
# (tests/test_flop_counts.py keeps these in step with it).
ALG_FLOPS = {2: 23601.0, 3: 356161.0, 4: 5744961.0, 5: 102333185.0}
# Flops per phase-space point the helicity-recycling matrix-element kernels
# execute (same counting convention): their stage functions run with the
# counting scalar (tests/test_flop_counts.py); the same for FP32 and FP64.
REC_FLOPS = {2: 4504.0, 3: 51648.0, 4: 675248.0, 5: 12509560.0}
# Bytes of the FP32 per-event record the g g > t t~ g g matrix-element kernel reads (PrepRec)
REC_BYTES = {4: 1536}
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12  # SMs x FP32 lanes x FMA x max clock
# DRAM bytes (read + write) of the g g > t t~ g g matrix-element kernel per
# passing event: one ncu capture of 10^6 points
# (profiles/me_rec_kernel_ggttxgg_mixed.md, 811.1 MB over 514,487 events);
# the kernel's traffic is its records, so it scales with the events of a launch
ME_DRAM_BYTES_PER_EVENT = 1576.0

C3_CUTS = dict(ptmin=60.0, etamax=2.5, drmin=0.4)
PDF = "synthetic gluon PDF x g=A x^-0.2 (1-x)^5 (100x50 bicubic), Q=mt"
CONFIGS = {
    "c1": dict(k=2, kind=0, sqrts=1000.0, cuts={}, events=1_000_000, iterations=5, precision="fp64",
               workload="g g > t t~ at fixed sqrt(s)=1 TeV, mt=173, wt=1.4915, alpha_s=0.118, 8-dim rambo, "
                        "no cuts, VEGAS 50 bins/dim",
               process="gg_ttx (3 diagrams, 2 colour flows, 16 helicities)"),
    "c2": dict(k=3, kind=1, sqrts=13000.0, cuts=dict(ptmin=30.0, etamax=4.0, drmin=0.0), events=10_000_000,
               iterations=10, precision="fp64",
               workload=f"g g > t t~ g, sqrt(S)=13 TeV, {PDF}, pT>30, |eta|<4, 14-dim ramboflow, VEGAS 50 bins/dim",
               process="gg_ttxg (16 diagrams, 6 colour flows, 32 helicities)"),
    "c3": dict(k=4, kind=1, sqrts=13000.0, cuts=C3_CUTS, events=10_000_000, iterations=10, precision="mixed",
               workload=f"g g > t t~ g g, sqrt(S)=13 TeV, {PDF}, pT>60, |eta|<2.5, dR(g,g)>0.4, "
                        "18-dim ramboflow, VEGAS 50 bins/dim",
               process="gg_ttxgg (123 diagrams, 24 colour flows, 64 helicities)"),
    "c5": dict(k=5, kind=1, sqrts=13000.0, cuts=C3_CUTS, events=1_000_000, iterations=10, precision="mixed",
               workload=f"g g > t t~ g g g, sqrt(S)=13 TeV, {PDF}, pT>60, |eta|<2.5, dR(g,g)>0.4, "
                        "22-dim ramboflow, VEGAS 50 bins/dim",
               process="gg_ttxggg (1240 diagrams, 120 colour flows, 128 helicities)"),
}
CONFIGS["c4"] = dict(CONFIGS["c3"], workload=CONFIGS["c3"]["workload"] + "; normalizing-flow proposal")
# p p > t t~ at leading order (madflow's first example): g g and the light
# q q~ / q~ q channels with synthetic quark densities beside the gluon
CONFIGS["pp"] = dict(k=2, kind=1, sqrts=13000.0, cuts={}, events=10_000_000, iterations=10, precision="mixed",
                     initial_states="pp",
                     workload=f"p p > t t~ (g g + q q~ + q~ q, q = d u s c), sqrt(S)=13 TeV, {PDF} and synthetic "
                              "quark densities, no cuts, 10-dim ramboflow, VEGAS 50 bins/dim",
                     process="gg_ttx (3 diagrams) + uux_ttx (1 diagram, 4 flavours and their mirror images)")
# p p > t t~ j at leading order: g g > t t~ g and the light-quark channels
# q q~ > t t~ g, q g > t t~ q, q~ g > t t~ q~ (and mirror images); the jet
# cuts of c2 on particle 4 whatever its flavour
CONFIGS["ppj"] = dict(k=3, kind=1, sqrts=13000.0, cuts=dict(ptmin=30.0, etamax=4.0, drmin=0.0), events=10_000_000,
                      iterations=10, precision="mixed", initial_states="pp",
                      workload=f"p p > t t~ j (g g > t t~ g + q q~ > t t~ g + q g > t t~ q + q~ g > t t~ q~, "
                               f"q = d u s c, mirror images), sqrt(S)=13 TeV, {PDF} and synthetic quark densities, "
                               "pT(j)>30, |eta(j)|<4, 14-dim ramboflow, VEGAS 50 bins/dim",
                      process="gg_ttxg (16 diagrams) + uux_ttxg, ug_ttxu, uxg_ttxux (5 diagrams each, one thread "
                              "per event, in the phase-space stage)")
KERNELS = {2: "ps_iter_kernel<2,{T},false> (phase space and |M|^2 in one pass)", 3: "me_rec_warp_kernel<3,{T}>", 4: "me_rec_kernel<4,{T},{C}>",
           5: "me_gws_kernel<5,{T},{C}>"}


def workload(cfg, events):
    return {"workload": cfg["workload"], "events_per_iteration": events, "process": cfg["process"]}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def measure_gemm_peak(dtype_name):
    """The SIMT pipe's rate as cuBLAS reaches it, measured in this run: an
    FP32 GEMM with TF32 off (8192^3) or an FP64 GEMM (4096^3), best of 5
    CUDA-event timings after 2 warm-ups."""
    import torch

    dt = torch.float32 if dtype_name == "fp32" else torch.float64
    n = 8192 if dt == torch.float32 else 4096
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        g = torch.Generator(device="cuda").manual_seed(0)
        a = torch.randn((n, n), dtype=dt, device="cuda", generator=g)
        b = torch.randn((n, n), dtype=dt, device="cuda", generator=g)
        for _ in range(2):
            c = a @ b
        best = float("inf")
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            c = a @ b
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b, c
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return 2.0 * n ** 3 / (best / 1000.0) / 1e12, f"cuBLAS {dtype_name.upper()} GEMM {n}^3 (TF32 off), best of 5"


def make_integrand(prec, cfg=None):
    from madflow_gb300.vegas import FusedIntegrand

    cfg = cfg or CONFIGS["c3"]
    return FusedIntegrand(cfg["k"], kind=cfg["kind"], sqrts=cfg["sqrts"], mt=MT, wt=WT, alpha_s=ALPHA_S,
                          precision=prec, initial_states=cfg.get("initial_states", "gg"), **cfg["cuts"])


def _prec_code(name):
    from madflow_gb300 import _lib

    return _lib.MF_PREC_MIXED if name == "mixed" else _lib.MF_PREC_FP64


def fused_steps(cfg, prec_name, N, steps, warmup, seed, dist=None, rank=0, local=0, sample_clocks=True,
                events_limit=None):
    """W untimed and K timed fused VEGAS iterations (L2 flushed before each),
    in slices of events_limit events if given; returns the timing record of
    the steps (stage times for one-slice steps only)."""
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.vegas import VegasFlow, reduce_results

    integ = make_integrand(_prec_code(prec_name), cfg)
    vegas = VegasFlow(integ.n_dim, N, seed=seed, stream_id=rank, use_graph=True)
    vegas.compile(integ)
    f_out = torch.empty(N, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    npass = torch.zeros(steps, dtype=torch.int64, device="cuda")

    def step():
        integ.iteration(vegas.grid, vegas.seed, vegas.stream_id, vegas.iteration, N, vegas.results, f_out=f_out,
                        events_limit=events_limit)
        if dist:
            # one grid over all ranks: the iteration sums are summed before the refinement
            reduce_results(vegas.results)
        _lib.call("mf_vegas_refine", vegas.grid.data_ptr(), vegas.results[2:].data_ptr(), vegas.n_dim, vegas.nbins,
                  vegas.alpha, torch.cuda.current_stream().cuda_stream)
        vegas.iteration += 1

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    # the pipeline records events between its stages (same stream), read after each step
    timing = events_limit is None or events_limit >= N
    integ.set_timing(timing)
    stage_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(steps):
            flush.zero_()
            starts[i].record()
            step()
            ends[i].record()
            npass[i] = torch.count_nonzero(f_out)
            ends[i].synchronize()
            if timing:
                stage_ms.append(integ.stage_ms())
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        wall = time.perf_counter() - t0
    integ.set_timing(False)
    nonfinite = integ.check_errors()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    return dict(integ=integ, step_s=sum(ms) / 1000.0, npass=[int(n) for n in npass.tolist()], stage_ms=stage_ms,
                wall=wall, clocks=clk.summary() if sample_clocks else None, nonfinite=nonfinite)


def run_gpu(args):
    import numpy as np
    import torch

    cfg = CONFIGS[args.config]
    k = cfg["k"]
    prec_name = args.precision or cfg["precision"]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    N = args.events or cfg["events"]
    # each rank draws its own Philox stream (stream id = rank); with several
    # ranks the iteration sums are all-reduced, so every rank refines one grid
    r = fused_steps(cfg, prec_name, N, args.steps, args.warmup, args.seed, dist, rank, local)
    integ = r["integ"]
    step_s = r["step_s"]
    n_me_rank = torch.tensor(sum(r["npass"]), dtype=torch.int64, device="cuda")
    if dist:
        t = torch.tensor([step_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_s = float(t.item())
        dist.all_reduce(n_me_rank)
    n_me = int(n_me_rank.item())
    pass_frac = n_me / (N * args.steps * world)
    me_per_s = n_me / step_s

    # dominant kernel: the matrix element; flops per launch = recycled flops
    # per event x the events passing the cuts, time from CUDA events on the
    # launching stream around the kernel
    # g g > t t~ evaluates |M|^2 in the phase-space pass (one thread per event)
    me_ms = [d["phase_space" if k == 2 else "matrix_element"] for d in r["stage_ms"]]
    achieved = REC_FLOPS[k] * sum(r["npass"]) / (sum(me_ms) / 1000.0) / 1e12
    stages = {s: statistics.mean(d[s] for d in r["stage_ms"]) for s in r["stage_ms"][0]}
    # the autotuner ran on the first (warm-up) iteration
    tune = integ.tuning()
    pipe = "fp32" if prec_name == "mixed" else "fp64"
    peak, peak_how = measure_gemm_peak(pipe)

    # end to end: the integrand contract f(x) on host buffers: the points in
    # page-locked host memory, read by the kernels over the host link, and f
    # written back to page-locked host memory (mf_integrand_rows, zero-copy);
    # the transfers run inside the timed call
    e2e_n = min(N, args.e2e_events)
    rng = np.random.default_rng(args.seed)
    x_host = torch.from_numpy(rng.uniform(size=(e2e_n, integ.n_dim))).pin_memory()
    f_host = torch.empty(e2e_n, dtype=torch.float64).pin_memory()
    integ(x_host, out=f_host)  # warm-up
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = max(1, args.e2e_reps)
    for _ in range(reps):
        integ(x_host, out=f_host)
    e1.record()
    torch.cuda.synchronize()
    # whole job: the passing events of all ranks over the slowest rank's time
    e2e_t = torch.tensor([e0.elapsed_time(e1) / 1000.0], dtype=torch.float64, device="cuda")
    e2e_pass = torch.tensor([int((f_host != 0).sum()) * reps], dtype=torch.int64, device="cuda")
    if dist:
        dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
        dist.all_reduce(e2e_pass)
    e2e_rate = int(e2e_pass.item()) / float(e2e_t.item())

    T = "float" if prec_name == "mixed" else "double"
    kern = KERNELS[k].format(T=T, C=tune["colour"] if prec_name == "mixed" else 0)
    traffic = None
    if k == 4 and prec_name == "mixed":
        traffic = ME_DRAM_BYTES_PER_EVENT * statistics.mean(r["npass"])
    out = {
        "metric": METRIC,
        "value": me_per_s,
        "unit": "|M|^2 evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * step_s / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (mixed: FP64 momenta, propagators, event weights, sums)" if prec_name == "mixed" else "f64",
        "data": "synthetic (Philox4x32-10 uniforms, seed %d)" % args.seed,
        "config": dict(workload(cfg, N), name=args.config, precision=prec_name,
                       l2="flushed (256 MB write) before every step",
                       parallelism=(f"sharded over {world} GPUs: own Philox stream and {N} points per rank, "
                                    "one NCCL all-reduce of the iteration sums per step, one grid")
                       if world > 1 else "single GPU"),
        "pass_fraction": pass_frac,
        "phase_space_points_per_s": N * args.steps * world / step_s,
        "wall_s": r["wall"],
        # per step: set-int, phase-space first pass, phase space, matrix element, accumulate, reduce, refine
        "gpu_launches": 7 * args.steps,
        "stage_ms": stages,
        "nonfinite_weights": r["nonfinite"],
        "autotune": dict(tune, variants="index colour*4 + log2(waves); colour 0 SIMT, 1 tensor cores (tcgen05 TF32)"),
        "e2e": {"value": e2e_rate, "unit": "|M|^2 evals/s", "h2d_bytes_per_step": int(x_host.numel() * 8) * world,
                "d2h_bytes_per_step": int(f_host.numel() * 8) * world,
                "api": "FusedIntegrand(x_host, out=f_host): x (N, ndim) float64 and f in page-locked host memory, "
                       "read and written by the kernels over the host link (mf_integrand_rows, zero-copy)",
                "events_per_step": e2e_n * world},
        "roofline": {"bound": pipe, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu, 10^6-point capture scaled by the events per launch)",
                     "algorithmic_bytes_per_event": REC_BYTES.get(k) if prec_name == "mixed" else None,
                     "kernel": kern,
                     "peak_source": f"measured in this run: {peak_how}" +
                                    (f"; nominal FP32 {FP32_NOMINAL_TFLOPS:.1f}" if pipe == "fp32" else ""),
                     "frac_of_nominal": achieved / FP32_NOMINAL_TFLOPS if pipe == "fp32" else None,
                     "flops_per_event": REC_FLOPS[k],
                     "alg_flops_per_event": ALG_FLOPS[k],
                     "alg_equivalent_tflops": achieved * ALG_FLOPS[k] / REC_FLOPS[k],
                     "kernel_ms": statistics.mean(me_ms)},
        "clocks": r["clocks"],
    }
    if rank == 0:
        extras(args, cfg, prec_name, out)
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def extras(args, cfg, prec_name, out):
    """The configuration's own measurements beside the throughput line."""
    k = cfg["k"]
    name = args.config
    if args.precision_points and cfg["k"] > 2:
        n = args.precision_points if k < 5 else min(args.precision_points, 100_000)
        out["mixed_vs_fp64"] = precision_study(cfg, n, args.seed + 2)
    if name in ("c1", "c2", "c5", "pp", "ppj") and args.integration:
        out["integration"] = {p: integration(cfg, p, cfg["events"], cfg["iterations"], args.seed + 5)
                              for p in (("fp64", "mixed") if name in ("c2", "pp", "ppj") else (prec_name,))}
        if name in ("pp", "ppj"):
            # the g g channel alone on the same points: the quark channels' share
            gg = integration(dict(cfg, initial_states="gg"), "mixed", cfg["events"], cfg["iterations"],
                             args.seed + 5)
            out["integration"]["gg_only_mixed"] = gg
            out["integration"]["qq_share"] = 1.0 - gg["result_pb"] / out["integration"]["mixed"]["result_pb"]
        if name == "c1":
            out["integration"]["oracle_replay"] = oracle_replay(cfg, cfg["events"], cfg["iterations"], args.seed + 5)
        if name == "c2":
            other = "mixed" if prec_name == "fp64" else "fp64"
            o = fused_steps(cfg, other, cfg["events"], 3, 2, args.seed, sample_clocks=False)
            out["other_precision"] = {"precision": other, "value": sum(o["npass"]) / o["step_s"],
                                      "unit": "|M|^2 evals/s", "ms_per_step": 1000.0 * o["step_s"] / 3}
    if name == "c3" and args.integration:
        # the same iteration in slices of events_limit events (scratch of one
        # slice): 10^6, and 5*10^4, the reference's own default for six
        # particles on a GPU with 13 GB or more (config.py:168-176)
        out["events_limit"] = {}
        for lim in (1_000_000, 50_000):
            o = fused_steps(cfg, prec_name, cfg["events"], 3, 2, args.seed, sample_clocks=False, events_limit=lim)
            out["events_limit"][str(lim)] = {"value": sum(o["npass"]) / o["step_s"], "unit": "|M|^2 evals/s",
                                             "ms_per_step": 1000.0 * o["step_s"] / 3,
                                             "scratch_bytes": o["integ"].scratch_bytes()}
    if name == "c3" and args.time_to_target:
        out["time_to_1e-3"] = time_to_target(args, cfg)
    if name == "c4":
        out["flow_vs_vegas"] = flow_vs_vegas(args, cfg)
    if name == "c5" and args.integration:
        out["flow_vs_vegas"] = flow_vs_vegas_budget(args, cfg)
    if args.cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, cfg)
        ttt = out.get("time_to_1e-3")
        if ttt and ttt.get("vegas_fp64", {}).get("events"):
            ev = ttt["vegas_fp64"]["events"] * ttt["vegas_fp64"]["pass_fraction"]
            cb = out["cpu_baseline"]
            cb["projected_seconds_to_1e-3"] = ev / cb["value"]
            cb["projection"] = ("the GPU FP64 VEGAS run's |M|^2 evaluations to 1e-3 (events x pass fraction) "
                                "divided by the measured CPU rate on this sample")
    if args.numpy_baseline:
        out["cpu_baseline_numpy"] = cpu_baseline_numpy(args, cfg)


def precision_study(cfg, n_events, seed):
    """|M|^2 and integrand error of the mixed-precision path against the FP64
    path (which agrees with the FP64 oracle to 1e-12) on the same fixed
    points: ramboflow momenta of n_events uniform points for |M|^2 (no cuts),
    the same points through the whole integrand with the configuration's cuts."""
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.matrix import PROCESSES
    from madflow_gb300.phasespace import ramboflow

    k = cfg["k"]
    gs = math.sqrt(4.0 * math.pi * ALPHA_S)
    coup = (complex(-gs, 0.0), complex(0.0, gs), complex(0.0, gs * gs))
    m64, m32 = PROCESSES[k](precision=_lib.MF_PREC_FP64), PROCESSES[k](precision=_lib.MF_PREC_MIXED)
    f64i, f32i = make_integrand(_lib.MF_PREC_FP64, cfg), make_integrand(_lib.MF_PREC_MIXED, cfg)
    g = torch.Generator(device="cuda").manual_seed(seed)
    chunk = 250_000 if k < 5 else 50_000
    rel, F64, F32 = [], [], []
    for s in range(0, n_events, chunk):
        x = torch.rand((min(chunk, n_events - s), 4 * k + 2), dtype=torch.float64, device="cuda", generator=g)
        p, *_ = ramboflow(x, k + 2, cfg["sqrts"], [MT, MT] + [0.0] * (k - 2))
        a = m64.smatrix(p, MT, WT, *coup)
        b = m32.smatrix(p, MT, WT, *coup)
        rel.append((b - a).abs() / a.abs())
        F64.append(f64i(x))
        F32.append(f32i(x))
    rel, F64, F32 = torch.cat(rel), torch.cat(F64), torch.cat(F32)
    qs = torch.tensor([0.5, 0.99, 0.999], dtype=torch.float64, device="cuda")
    q = torch.quantile(rel, qs).tolist()
    same = (F64 == 0) == (F32 == 0)
    both = same & (F64 != 0)
    a, b = F64[both], F32[both]
    frel = (b - a).abs() / a.abs()
    fq = torch.quantile(frel, qs).tolist()
    return {"points": n_events,
            "me_rel_err": {"median": q[0], "p99": q[1], "p999": q[2], "max": float(rel.max())},
            "integrand_rel_err": {"median": fq[0], "p99": fq[1], "p999": fq[2], "max": float(frel.max()),
                                  "xsec_share_err_gt_1e-3": float(a[frel > 1e-3].abs().sum() / a.abs().sum()),
                                  "l1": float((b - a).abs().sum() / a.abs().sum()),
                                  "sum": float(abs(F32[same].sum() - F64[same].sum()) / F64[same].abs().sum()),
                                  "cut_decisions_differing": int((~same).sum())},
            "momenta": f"ramboflow of uniform points, sqrt(S) = {cfg['sqrts']:g} GeV, no cuts (|M|^2); "
                       "the integrand with the configuration's cuts"}


def integration(cfg, prec_name, n_events, iterations, seed):
    """`iterations` fused VEGAS iterations from a uniform grid (wall clock,
    first iteration included, after an untimed warm-up call that runs the
    launch autotuner and allocates the scratch)."""
    import torch

    from madflow_gb300.vegas import VegasFlow

    integ = make_integrand(_prec_code(prec_name), cfg)
    warm = min(n_events, 262_144)
    integ(torch.rand((warm, integ.n_dim), dtype=torch.float64, device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(1)))
    v = VegasFlow(integ.n_dim, n_events, seed=seed, use_graph=True)
    v.compile(integ)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res, err = v.run_integration(iterations)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"result_pb": res, "error_pb": err, "rel_error": err / abs(res) if res else None, "seconds": dt,
            "iterations": iterations, "events_per_iteration": n_events,
            "per_iteration": [{"result_pb": a, "error_pb": b} for a, b, _ in v.last_run]}


def oracle_replay(cfg, n_events, iterations, seed):
    """The oracle's VEGAS (Lepage) over the same Philox uniforms and grid
    updates, FP64 on the CPU: the same samples, so the integral agrees far
    inside the statistical error."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    ndim, nb = 8, 50
    grid = np.tile(np.linspace(0.0, 1.0, nb + 1), (ndim, 1))
    ocfg = [cfg["kind"], cfg["k"], cfg["sqrts"], MT, WT, ALPHA_S, 0.0, 0.0, 0.0, 0]
    wsum = wres = 0.0
    t0 = time.perf_counter()
    for it in range(iterations):
        u = oracle.uniforms(seed, 0, it, 0, n_events, ndim)
        x, jac, bins = oracle.vegas_sample(grid, u)
        f = oracle.integrand(ocfg, x, fast=True)
        sums, hist = oracle.vegas_accumulate(f * jac / n_events, bins, nb)
        var = (n_events * sums[1] - sums[0] ** 2) / (n_events - 1.0)
        wsum += 1.0 / var
        wres += sums[0] / var
        grid = oracle.vegas_refine(grid, hist, 1.5)
    return {"result_pb": wres / wsum, "error_pb": 1.0 / math.sqrt(wsum), "seconds": time.perf_counter() - t0,
            "cores": oracle.num_threads(True)}


def _vegas_to_target(cfg, prec, n_events, seed, max_iter, target):
    import torch

    from madflow_gb300.vegas import VegasFlow

    integ = make_integrand(prec, cfg)
    # untimed warm-up: the launch autotuner (first call with >= 262144 points) and the allocations
    integ(torch.rand((262_144, integ.n_dim), dtype=torch.float64, device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(1)))
    v = VegasFlow(integ.n_dim, n_events, seed=seed, use_graph=True)
    v.compile(integ)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res, err = v.run_integration(max_iter, target_rel_error=target)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    it = len(v.last_run)
    return {"seconds": dt, "iterations": it, "events_per_iteration": n_events, "events": it * n_events,
            "result_pb": res, "error_pb": err, "rel_error": err / abs(res) if res else None,
            "reached": bool(res and err / abs(res) <= target), "vegas": v,
            "untimed_warmup": "one integrand call of 262144 points (launch autotuner, allocations)"}


def _public(d):
    return {a: b for a, b in d.items() if a != "vegas"}


def _flow(args, integ, layers, bins, bf16):
    """bf16: False (TF32 tensor-core sampling), "tc" (BF16 tensor-core
    sampling, both hand-written; training in the FP32 layer kernels) or True
    (BF16 GEMMs through torch autocast / cuBLAS)."""
    from madflow_gb300.flow import NormalizingFlow

    if bf16 == "tc":
        return NormalizingFlow(integ.n_dim, n_layers=layers, bins=bins, hidden=args.flow_hidden, n_hidden=2, seed=0,
                               tc_bf16=True)
    return NormalizingFlow(integ.n_dim, n_layers=layers, bins=bins, hidden=args.flow_hidden, n_hidden=2, seed=0,
                           bf16=bf16, tf32=not bf16)


def _flow_kernels(flow):
    if flow.bf16:
        return "BF16 GEMMs with FP32 accumulation (torch autocast, cuBLAS) and the hand-written transform kernels"
    train = "training in the hand-written FP32 layer kernels" if flow.native else "training through torch/cuBLAS"
    sample = (f"sampling in one tcgen05 {'BF16' if flow.tc_bf16 else 'TF32'} kernel per layer" if flow.fused else
              "sampling in the hand-written FP32 layer kernels" if flow.native else "sampling through torch/cuBLAS")
    return f"{sample}, {train}"


def _flow_leg(args, integ, target, layers, bins, bf16, vegas_iters, vegas_events, batch, train_batches,
              max_batches):
    """A few VEGAS iterations adapt a grid, then the flow refines the proposal
    on top of the frozen grid (all inside the timed region).  Every VEGAS
    iteration and flow batch is an unbiased estimate; they are combined with
    inverse-variance weights."""
    import torch

    from madflow_gb300.flow import adaptive_flow_integration
    from madflow_gb300.vegas import VegasFlow

    def run(flow, grid, prior, target_, max_b, train_b):
        return adaptive_flow_integration(flow, integ, target_rel_error=target_, batch_size=batch,
                                         max_batches=max_b, lr=args.flow_lr, train_batches=train_b,
                                         minibatch=args.flow_minibatch, grid=grid, prior=prior,
                                         resample=args.flow_resample, train_steps=args.flow_train_steps)

    # untimed warm-up of the flow's kernels and GEMM shapes, the launch autotuner and the allocations
    run(_flow(args, integ, layers, bins, bf16), None, None, 0.0, 2, 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    v = VegasFlow(integ.n_dim, vegas_events, seed=args.seed + 2, use_graph=True)
    v.compile(integ)
    vr, ve = v.run_integration(vegas_iters)
    flow = _flow(args, integ, layers, bins, bf16)
    t_flow = time.perf_counter()
    res, err, info = run(flow, v.grid, (1.0 / ve ** 2, vr / ve ** 2), target, max_batches, train_batches)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    dt = t1 - t0
    return {"seconds": dt, "vegas_seconds": t_flow - t0, "flow_seconds": t1 - t_flow,
            "vegas_iterations": vegas_iters, "vegas_events_per_iteration": vegas_events,
            "flow_batches": info["batches"], "trained_batches": info["trained"], "events_per_batch": batch,
            "events": info["batches"] * batch + vegas_iters * vegas_events,
            "result_pb": res, "error_pb": err, "rel_error": err / abs(res) if res else None,
            "reached": bool(res and err / abs(res) <= target),
            "flow": f"{layers} piecewise-quadratic coupling layers, {bins} bins, MLP 2x{args.flow_hidden} "
                    f"({_flow_kernels(flow)}), "
                    f"lr {args.flow_lr}, on a frozen VEGAS grid, trained on {args.flow_resample} events per batch "
                    f"resampled with probability w^2 ({args.flow_train_steps} Adam step(s) per batch, each on its "
                    "own resample, a captured CUDA graph)",
            "last_std_over_mean": info["last_rel_std"]}, flow, v.grid


def time_to_target(args, cfg, target=1e-3):
    """Wall-clock seconds until the combined relative error of the integral
    reaches the target, from a fresh start (uniform grid / untrained flow):
    plain VEGAS in FP64 (the reference's arithmetic), VEGAS in mixed
    precision, and the normalizing-flow sampler in mixed precision."""
    import torch

    from madflow_gb300 import _lib

    out = {"target_rel_error": target}
    out["vegas_fp64"] = _public(_vegas_to_target(cfg, _lib.MF_PREC_FP64, args.target_events, args.seed + 1,
                                                 args.max_iter, target))
    out["vegas_mixed"] = _public(_vegas_to_target(cfg, _lib.MF_PREC_MIXED, args.target_events, args.seed + 1,
                                                  args.max_iter, target))
    integ = make_integrand(_lib.MF_PREC_MIXED, cfg)
    # pass fraction of the workload (for the CPU projection)
    x = torch.rand((200_000, integ.n_dim), dtype=torch.float64, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(7))
    out["vegas_fp64"]["pass_fraction"] = float((integ(x) != 0).double().mean())
    out["flow_mixed"] = _flow_leg(args, integ, target, args.flow_layers, args.flow_bins, args.flow_bf16,
                                  args.flow_vegas_iters, args.flow_vegas_events, args.flow_batch,
                                  args.flow_train_batches, args.max_iter * 4)[0]
    return out


def _unweighting_efficiency(w):
    """<w> / w_max of a weighted sample, w_max truncated so that at most 1e-3
    of the cross section sits above it (as the LHE writer unweights), and the
    untruncated <w> / max w."""
    from madflow_gb300.lhe import truncated_wmax

    w = w.abs()
    mean = float(w.mean())
    return {"truncated_1e-3": mean / truncated_wmax(w, 1e-3), "untruncated": mean / float(w.max()),
            "events": int(w.numel())}


def _sample_vegas(integ, grid, n, seed):
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.config import stream_ptr
    from madflow_gb300.flow import _vegas_map

    u = torch.empty((integ.n_dim, n), dtype=torch.float64, device="cuda")
    _lib.call("mf_philox_uniforms", seed, 9, 0, 0, n, integ.n_dim, u.data_ptr(), stream_ptr())
    x, jac = _vegas_map(grid, u.T.contiguous())
    return integ(x) * jac


def _sample_flow(integ, flow, grid, n, seed):
    import torch

    from madflow_gb300.flow import _clamp_open, _vegas_map

    z, logq = flow.sample(n, seed=seed, iteration=999)
    z = _clamp_open(z)
    x, jac = _vegas_map(grid, z)
    return integ(x) * jac * torch.exp(-logq)


def flow_vs_vegas(args, cfg, target=1e-3):
    """The c3 integrand with the configuration's flow (6 coupling layers, 16
    bins, MLP 2 x 64, BF16 GEMMs, 20 training batches of 10^6 events) against
    plain VEGAS at 10^6 events per iteration: time and events to the target,
    and the unweighting efficiency of the final proposal on 10^6 events."""
    from madflow_gb300 import _lib

    integ = make_integrand(_lib.MF_PREC_MIXED, cfg)
    n = 1_000_000
    vg = _vegas_to_target(cfg, _lib.MF_PREC_MIXED, n, args.seed + 1, args.max_iter * 4, target)
    out = {"target_rel_error": target, "vegas": _public(vg)}
    out["vegas"]["unweighting_efficiency"] = _unweighting_efficiency(_sample_vegas(integ, vg["vegas"].grid, n, 77))
    # the configuration's flow: hand-written FP32 training with TF32 or BF16
    # tensor-core sampling, and with its BF16 GEMMs through cuBLAS
    for key, bf16 in (("flow", False), ("flow_bf16", "tc"), ("flow_bf16_cublas", True)):
        fl, flow, grid = _flow_leg(args, integ, target, 6, 16, bf16, args.flow_vegas_iters, args.flow_vegas_events,
                                   n, 20, args.max_iter * 4)
        fl["unweighting_efficiency"] = _unweighting_efficiency(_sample_flow(integ, flow, grid, n, 78))
        out[key] = fl
    return out


def flow_vs_vegas_budget(args, cfg, budget_iters=10):
    """g g > t t~ g g g at 10^6 events per iteration: plain VEGAS against the
    flow proposal (c4 architecture on top of a VEGAS grid of 3 iterations),
    each for the same total number of events; relative error reached, time
    and unweighting efficiency."""
    import torch

    from madflow_gb300 import _lib
    from madflow_gb300.vegas import VegasFlow

    integ = make_integrand(_lib.MF_PREC_MIXED, cfg)
    n = 1_000_000
    integ(torch.rand((20_000, integ.n_dim), dtype=torch.float64, device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(1)))
    v = VegasFlow(integ.n_dim, n, seed=args.seed + 1, use_graph=True)
    v.compile(integ)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res, err = v.run_integration(budget_iters)
    torch.cuda.synchronize()
    out = {"events": budget_iters * n,
           "vegas": {"seconds": time.perf_counter() - t0, "result_pb": res, "error_pb": err,
                     "rel_error": err / abs(res) if res else None,
                     "unweighting_efficiency": _unweighting_efficiency(_sample_vegas(integ, v.grid, n, 77))}}
    vi = 3
    fl, flow, grid = _flow_leg(args, integ, 0.0, 6, 16, False, vi, n, n, budget_iters - vi, budget_iters - vi)
    fl["unweighting_efficiency"] = _unweighting_efficiency(_sample_flow(integ, flow, grid, n, 78))
    out["flow"] = fl
    return out


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def cpu_baseline(args, cfg, sample=None):
    """The CPU restatement of madflow's integrand (the oracle, C++/OpenMP over
    all host cores, timing build) on a bounded sample of the same workload."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    k = cfg["k"]
    n = sample or args.cpu_events
    if k == 5 and sample is None:
        n = max(1000, n // 20)
    plan = oracle.TTNG(k, fast=True)
    ndim = 8 if cfg["kind"] == 0 else 4 * k + 2
    rng = np.random.default_rng(args.seed)
    x = rng.uniform(size=(n, ndim))
    c = cfg["cuts"]
    ocfg = [cfg["kind"], k, cfg["sqrts"], MT, WT, ALPHA_S, c.get("ptmin", 0.0), c.get("etamax", 0.0),
            c.get("drmin", 0.0), 0, 1 if cfg.get("initial_states") == "pp" else 0]
    oracle.integrand(ocfg, x[: min(256, n)], plan)  # warm-up
    t0 = time.perf_counter()
    f = oracle.integrand(ocfg, x, plan)
    dt = time.perf_counter() - t0
    n_me = int((f != 0).sum())
    return {"value": n_me / dt, "unit": "|M|^2 evals/s", "cores": oracle.num_threads(True), "kind": "port",
            "sample": f"{n} phase-space points of the same workload ({n_me} pass the cuts), {dt:.1f} s",
            "seconds": dt, "events": n_me, "cpu": _cpu_model(), "machine": platform.machine(),
            "build": f"g++ {oracle.FAST_FLAGS} (oracle/Makefile timing build; no -march=native, so the same "
                     "flags build on x86-64 and Arm)",
            "algorithm": "madflow's FP64 per-event evaluation: every helicity separately, dense colour sum"}


def cpu_baseline_numpy(args, cfg):
    """The vectorised NumPy FP64 restatement (oracle/np_ref.py: [6, N]
    complex arrays over the event axis, every helicity separately, madflow's
    CPU array style) timed on |M|^2 of a bounded sample of the workload's
    momenta (ramboflow of uniform points, the events that pass the cuts)."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import np_ref
    import oracle

    oracle.build()
    k = cfg["k"]
    rng = np.random.default_rng(args.seed)
    x = rng.uniform(size=(4 * args.numpy_events, 4 * k + 2))
    p, *_, x1, x2 = oracle.ramboflow(x, k + 2, cfg["sqrts"], [MT, MT] + [0.0] * (k - 2))
    lab = oracle.boost_to_lab(p, x1, x2)
    c = cfg["cuts"]
    keep = [e for e in range(len(lab)) if oracle.pass_cuts(lab[e], c.get("ptmin", 0.0), c.get("etamax", 0.0),
                                                           c.get("drmin", 0.0))]
    p = p[keep[: args.numpy_events]]
    plan = np_ref.TTNG(k, oracle.TTNG(k).colour)
    gs = float(np.sqrt(4 * np.pi * ALPHA_S))
    plan.smatrix(p[:64], MT, WT, -gs, 1j * gs, 1j * gs * gs)  # warm-up
    t0 = time.perf_counter()
    plan.smatrix(p, MT, WT, -gs, 1j * gs, 1j * gs * gs)
    dt = time.perf_counter() - t0
    return {"value": len(p) / dt, "unit": "|M|^2 evals/s", "cores": 1, "kind": "port",
            "sample": f"{len(p)} passing events of the workload, |M|^2 only, {dt:.1f} s", "seconds": dt,
            "cpu": _cpu_model()}


def run_reference(args):
    """The reference arm: madflow's CPU path (its FP64 algorithm restated in
    C++/OpenMP, timing build, all host cores), W warm-up and K timed steps,
    each step a bounded sample of the same workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = CONFIGS[args.config]
    # five gluons cost ~20 times four per event: a proportionally smaller sample
    n_ref = args.ref_events if cfg["k"] < 5 else max(1000, args.ref_events // 20)
    for _ in range(args.warmup):
        cpu_baseline(args, cfg, 2000 if cfg["k"] < 5 else 200)
    steps = [cpu_baseline(args, cfg, n_ref) for _ in range(args.steps)]
    secs = sum(s["seconds"] for s in steps)
    n_me = sum(s["events"] for s in steps)
    value = n_me / secs
    cb = dict(steps[0])
    cb.update(value=value, seconds=secs,
              sample=f"{args.steps} steps x {n_ref} phase-space points of the same workload "
                     f"({n_me} pass the cuts), {secs:.1f} s")
    out = {
        "metric": METRIC,
        "value": value,
        "unit": cb["unit"],
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * secs / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (uniform points, seed %d)" % args.seed,
        "config": dict(workload(cfg, args.events or cfg["events"]), name=args.config),
        "impl": "reference",
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": cb["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def launch_ranks(args):
    """--gpus N > 1 without a torchrun environment: start N ranks (one per
    GPU) through torch.distributed.run on 127.0.0.1 and return its exit code."""
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", choices=sorted(CONFIGS), default="c3")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--events", type=int, default=0, help="points per iteration (default: the configuration's)")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default=None,
                    help="default: the configuration's (c1, c2 fp64; c3, c4, c5 mixed)")
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-events", type=int, default=200_000)
    ap.add_argument("--ref-events", type=int, default=40_000)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--numpy-baseline", action="store_true",
                    help="also time the vectorised NumPy restatement (one core; slow, off by default)")
    ap.add_argument("--numpy-events", type=int, default=3000)
    ap.add_argument("--no-time-to-target", dest="time_to_target", action="store_false")
    ap.add_argument("--no-integration", dest="integration", action="store_false")
    ap.add_argument("--target-events", type=int, default=4_000_000)
    ap.add_argument("--max-iter", type=int, default=40)
    ap.add_argument("--flow-layers", type=int, default=4)
    ap.add_argument("--flow-bins", type=int, default=8)
    ap.add_argument("--flow-bf16", action="store_true", help="bf16 MLP GEMMs (default TF32)")
    ap.add_argument("--flow-hidden", type=int, default=64)
    ap.add_argument("--flow-batch", type=int, default=1_000_000)
    ap.add_argument("--flow-minibatch", type=int, default=200_000)
    ap.add_argument("--flow-resample", type=int, default=50_000)
    ap.add_argument("--flow-lr", type=float, default=1e-2)
    ap.add_argument("--flow-train-batches", type=int, default=20)
    ap.add_argument("--flow-train-steps", type=int, default=1, help="optimiser steps per trained flow batch")
    ap.add_argument("--flow-vegas-iters", type=int, default=5)
    ap.add_argument("--flow-vegas-events", type=int, default=2_000_000)
    ap.add_argument("--precision-points", type=int, default=1_000_000)
    ap.add_argument("--e2e-events", type=int, default=4_000_000)
    ap.add_argument("--e2e-reps", type=int, default=3)
    return ap.parse_args(argv)


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "0"))
    if args.gpus > 1 and world == 0:
        sys.exit(launch_ranks(args))
    if world and world != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
