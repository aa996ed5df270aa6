"""Benchmark of viltrum's per-bin integration path on GB300.

Workload (one "step"): per-bin adaptive nested Newton-Cotes, nested(boole, simpson) with the default
absolute-error heuristic and 15 splits per bin (16 regions per bin), over 512x512 bins of the
synthetic scene "64 Gaussian bumps + 32 hard-edged disks" (SplitMix64 seed 7) on [0,1]^2 --
integrator_per_bin_parallel(integrator_adaptive_iterations(nested(boole,simpson), 15)).

Metric: integrand evaluations per second (Gsamples/s) of the whole step, kernel-only with the
scene resident on the device (`value`), and end to end through the public API with host buffers
(`e2e`: the step's input -- the scene parameters -- copied from pinned host memory, and the 512x512
bin image read back to pinned host memory, inside the timed region).  The bin RMSE of the result
against the FP64 closed-form bin integrals is reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU path (the oracle's restatement, which
reproduces the reference bit for bit; the reference itself cannot be built on the GPU host) on all
host cores over a bounded sample of bins per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms to bin RMSE 1e-3 vs FP64 oracle (learned-CV vs plain GPU); Gsamples/s"
RES = [512, 512]
ITERS = 15
SEED = 7
# integrand cost per evaluation of the scene, in FP32 flops (FMA = 2): per Gaussian bump
# 2 sub + mul + fma + mul + exp(mul + 3 fma + 7 fma + 2 mul) + fma = 31; per disk sub, sub, mul,
# fma, compare (+ add) = 6
FLOPS_PER_EVAL = 64 * 31 + 32 * 6


def culled_flops_per_eval(params, rmin, rmax, res) -> float:
    """Mean FP32 flops of one evaluation when only the scene's terms that can be non-zero in the
    evaluated bin are summed (the kernel's culled evaluation: a bump whose exponent is -87 or below
    over the whole bin adds exactly 0, as does a disk that misses the bin), averaged over the bins;
    per-term costs as in FLOPS_PER_EVAL.  The kernel culls over the box of the few consecutive bins
    of a warp, so it executes slightly more than this."""
    p = np.asarray(params, np.float32)
    ng, nd = int(p[0]), int(p[1])
    g = p[2:2 + 4 * ng].reshape(ng, 4).astype(np.float64)
    d = p[2 + 4 * ng:2 + 4 * ng + 4 * nd].reshape(nd, 4).astype(np.float64)
    edges = [rmin[k] + np.arange(res[k] + 1) * (rmax[k] - rmin[k]) / res[k] for k in range(2)]

    def gap(c, k):  # distance from c to each bin interval along dimension k
        lo, hi = edges[k][:-1], edges[k][1:]
        return np.maximum(np.maximum(lo - c, c - hi), 0.0)
    kept_g = np.zeros((res[1], res[0]))
    for cx, cy, sg, _ in g:
        d2 = gap(cy, 1)[:, None] ** 2 + gap(cx, 0)[None, :] ** 2
        kept_g += d2 * (0.5 / (sg * sg)) <= 87.0
    kept_d = np.zeros((res[1], res[0]))
    for cx, cy, r, _ in d:
        d2 = gap(cy, 1)[:, None] ** 2 + gap(cx, 0)[None, :] ** 2
        kept_d += d2 <= r * r
    return float(np.mean(kept_g * 31 + kept_d * 6))


def _peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def stripe(rank: int, world: int):
    """rank r integrates the horizontal stripe y in [r/world, (r+1)/world] with its own RES bins
    (weak scaling: every rank does one full workload, no data exchange)."""
    return [0.0, rank / world], [1.0, (rank + 1) / world]


def max_over_ranks(value: float, device: str = "cuda") -> float:
    """the largest of every rank's value (the job's time is its slowest rank's)"""
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args) -> dict | None:
    import torch

    import viltrum_gb300 as v
    from viltrum_gb300 import _lib, scenes

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    ctx = v.Context(local, stream=stream.cuda_stream)
    params = scenes.scene2(SEED)
    rmin, rmax = stripe(rank, ws)
    nb = RES[0] * RES[1]
    nested = _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)
    dev_bins = torch.empty(nb, dtype=torch.float32, device="cuda")
    p_dev = ctx.problem(scenes.SCENE2, params, rmin, rmax, RES, mem=_lib.MEM_DEVICE)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def step():
        return ctx.per_bin_adaptive_nested(p_dev, nested, ITERS, dev_bins)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    evals = 0
    launches = 0
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.fill_(i & 0xFF)  # evict the previous step's bins from L2 (outside the timed events)
            starts[i].record(stream)
            st = step()
            stops[i].record(stream)
            evals += st.evaluations
            launches += st.kernel_launches
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, stops)]
    total_ms = float(sum(step_ms))
    if ws > 1:
        total_ms = max_over_ranks(total_ms)
    value = evals * ws / (total_ms * 1e-3) / 1e9

    # accuracy of this step's result against the FP64 closed-form bin integrals
    out = dev_bins.cpu().numpy()
    exact = scenes.exact_bins(scenes.SCENE2, params, rmin, rmax, RES)
    rmse = scenes.bin_rmse(out.reshape(-1, 1), exact)

    # end to end through the public API: pinned host input and output buffers
    params_host = torch.from_numpy(params).pin_memory()
    bins_host = torch.empty(nb, dtype=torch.float32).pin_memory()
    bins_np = bins_host.numpy()
    integrator = v.integrator_per_bin_parallel(v.integrator_adaptive_iterations(
        v.nested(v.boole, v.simpson), v.error_heuristic_default(v.error_metric_absolute()), ITERS))
    rng = v.Range(rmin, rmax)
    e2e_value = None
    if not args.no_e2e:
        for _ in range(max(1, args.warmup)):
            v.integrate_into(integrator, bins_np, RES, v.Integrand.scene2(params_host.numpy()), rng, ctx=ctx,
                             device_bins=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v.integrate_into(integrator, bins_np, RES, v.Integrand.scene2(params_host.numpy()), rng, ctx=ctx,
                             device_bins=False)
        e2e_s = time.perf_counter() - t0
        e2e_value = round(evals * ws / e2e_s / 1e9, 4)

    # roofline of the dominant kernel (the nested-quadrature kernel is the only kernel of a step)
    peaks = _peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s
    per_launch_ms = total_ms / args.steps
    flops_eval = culled_flops_per_eval(params, rmin, rmax, RES)
    achieved = (evals / args.steps) * flops_eval / (per_launch_ms * 1e-3) / 1e12
    traffic = _traffic_from_profile(nb)
    line = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "Gsamples/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: 64 Gaussian bumps + 32 disks drawn by SplitMix64 (seed 7); FP64 truth from closed forms",
        "config": {
            "workload": "per-bin adaptive nested Newton-Cotes: nested(boole,simpson), default absolute heuristic, "
                        f"15 splits (16 regions) per bin, {RES[0]}x{RES[1]} bins of the 2-D scene",
            "bins": RES, "regions_per_bin": ITERS + 1, "evaluations_per_step": evals // args.steps,
            "l2": "flushed between timed steps by a 256 MiB device write outside the timed events",
            "parallelism": f"replicas: {ws} rank(s), one stripe of the image each",
        },
        "rmse_vs_fp64": rmse,
        "rel_rmse_vs_fp64": rmse / float(np.sqrt(np.mean(exact ** 2))),
        "roofline": {
            "bound": "fp32", "achieved": round(achieved, 3), "peak": round(fp32_peak, 3), "unit": "TFLOP/s",
            "frac": round(achieved / fp32_peak, 4), "traffic": traffic,
            "peak_source": "nominal FP32 FMA rate, 152 SMs x 128 lanes x 2 flop x sm_max_mhz of MEASURED_PEAKS.json "
                           "(that file holds no FP32 figure; the kernel moves ~1 MB per launch, so HBM is not its bound)",
            "flops_per_evaluation": round(flops_eval, 1),
            "flops_per_evaluation_unculled": FLOPS_PER_EVAL,
            "flops_note": "achieved counts the flops of the terms that can be non-zero in each bin (the culled "
                          "evaluation the kernel runs; every result equals the full sum bit for bit)",
        },
        "e2e": {"value": e2e_value, "unit": "Gsamples/s", "h2d_bytes_per_step": int(params.nbytes),
                "d2h_bytes_per_step": int(nb * 4)},
        "clocks": clocks.summary(),
        "gpu_launches": launches,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    if rank == 0 and ws == 1 and not args.no_configs:
        line["configs"] = other_configs(ctx, args)
        # the metric's first half: time to bin RMSE 1e-3 on the 5-D occluded scene at 1024x1024
        ttr = line["configs"].get("learned_vs_plain", {})
        case = next((v for k, v in ttr.items() if k.startswith("occluded_scene5")), None)
        if case:
            line["time_to_rmse"] = {
                "target_rmse": ttr.get("target_rmse"), "bins": case.get("bins"), "seeds": ttr.get("seeds"),
                "plain_mc_ms": case["plain_mc"]["mean_ms"], "polynomial_cv_ms": case["polynomial_cv"]["mean_ms"],
                "learned_cv_ms": case["learned_cv"]["mean_ms"],
                "learned_over_plain_ms": case.get("learned_over_plain_ms"),
                "learned_over_polynomial_ms": case.get("learned_over_polynomial_ms"),
                "higher_is_better": False}
    ctx.close()
    if ws > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


def _median_ms(fn, reps: int = 5, warmup: int = 3) -> tuple[float, object]:
    """median device time (the library's CUDA-event stats) of fn() after warm-up calls"""
    for _ in range(warmup):
        fn()
    out = [fn() for _ in range(reps)]
    return statistics.median(o.device_ms for o in out), out[-1]


def other_configs(ctx, args) -> dict:
    """One measured line per remaining workload of the path (rank 0, one GPU): per-bin Monte Carlo,
    control variates, the batch of independent integrals and the learned control variate against
    plain Monte Carlo and the polynomial control variate at equal bin RMSE."""
    from viltrum_gb300 import _lib, scenes

    out = {}
    # -- per-bin Monte Carlo, sin(8x)e^-y + x^2 + y^2 into 1024 bins along x, 1024 samples per bin
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [1024])
    b = np.empty(1024, np.float32)
    ms, st = _median_ms(lambda: ctx.per_bin_monte_carlo(p, 1024, 1, b))
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], [1024])
    from oracle import oracle as orc
    port = orc.port()
    t0 = time.perf_counter()
    port.per_bin_monte_carlo(scenes.WAVE2, None, [0, 0], [1, 1], [1024], 1024, 1)
    cpu_s = time.perf_counter() - t0
    out["per_bin_monte_carlo"] = {
        "workload": "wave2 sin(8x)e^-y+x^2+y^2 on [0,1]^2, 1024 bins along x, 1024 Philox samples per bin",
        "ms": round(ms, 4), "gsamples_s": round(st.evaluations / (ms * 1e6), 3),
        "rmse_vs_fp64": scenes.bin_rmse(b.reshape(-1, 1), exact), "timing": "median of 5 after 3 warm-up, device",
        "cpu_baseline": {"ms": round(cpu_s * 1e3, 2), "gsamples_s": round(1024 * 1024 / cpu_s / 1e9, 4), "cores": 1,
                         "kind": "port", "sample": "the whole workload (the reference's per-bin mt19937 path)"}}
    # -- control variates + residual Monte Carlo, 3 channels, 512x512 bins, 2^14 regions, 64 spp
    params = scenes.moving_scene3(SEED)
    res = [512, 512]
    p = ctx.problem(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res)
    nested = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
    b = np.empty(512 * 512 * 3, np.float32)
    ms, st = _median_ms(lambda: ctx.control_variates(p, nested, (1 << 14) - 1, _lib.CvOpts(64, 3, 0, 0, 1.0), b),
                        reps=3, warmup=3)
    rows = list(range(0, 512, 64))
    err = []
    for r in rows:
        y0, y1 = r / 512.0, (r + 1) / 512.0
        # one row of bins: its values are prod(res) x integral, and this call's resolution is [512, 1]
        ex = scenes.exact_bins(scenes.MOVING_SCENE3, params, [0, y0, 0], [1, y1, 1], [512, 1]) * 512.0
        err.append(b.reshape(512, 512, 3)[r] - ex)
    err = np.concatenate(err)
    t0 = time.perf_counter()
    port.control_variates(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], [128, 128],
                          orc.Nested.make("simpson", "trapezoidal", "size", "relative"), (1 << 14) - 1, 64, 3)
    cv_cpu_s = time.perf_counter() - t0
    out["control_variates"] = {
        "workload": "integrator_crespo2021(2^14-1 splits, 64 residual samples): moving-disk scene, RGB, "
                    "x,y binned 512x512, t in [0,1]",
        "ms": round(ms, 3), "gsamples_s": round(st.evaluations / (ms * 1e6), 3), "regions": int(st.regions),
        "rmse_vs_fp64": float(np.sqrt(np.mean(err.astype(np.float64) ** 2))),
        "rmse_sample": f"{len(rows)} of 512 rows of bins", "timing": "median of 3 after 3 warm-up, device",
        "cpu_baseline": {"ms_128x128": round(cv_cpu_s * 1e3, 1), "cores": 1, "kind": "port",
                         "sample": "the same regions (2^14-1 splits) and 64 samples/bin over 128x128 bins (1/16 of "
                                   "the bins; the residual part scales with the bins)"}}
    # -- batch of 4096 independent integrals (dims 2-6, budgets 256..65536, MC or nested)
    items = scenes.batch_items(4096, seed=11)
    prep = _lib.batch_items(items)
    st_nested = _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37)
    r, st, rep = ctx.integrate_batch(scenes.HALFSPACE, prep, st_nested)  # first call: layout + autotune
    item_ms = np.zeros(4096, np.float32)
    runs = [ctx.integrate_batch_resident(r, item_ms=item_ms) for _ in range(3)]
    ms = statistics.median(s_.device_ms for s_, _ in runs)
    t0 = time.perf_counter()
    for _ in range(2):
        ctx.integrate_batch(scenes.HALFSPACE, prep, st_nested, results=r)
    e2e_ms = (time.perf_counter() - t0) / 2 * 1e3
    # the reference's per-item CPU path on all host threads over 64 random items of the batch (items of
    # at most 3 M evaluations, so that the sample stays within seconds)
    import concurrent.futures as cf
    import random

    def evals_of(it):
        return it["budget"] if it["method"] == 0 else 3 ** it["dim"] + (it["budget"] - 1) * 2 * 3 ** (it["dim"] - 1)

    small = [i for i, it in enumerate(items) if evals_of(it) <= 3_000_000]
    pick = random.Random(1).sample(small, 64)
    nst_o = orc.Nested.make("simpson", "trapezoidal")

    def one(i):
        it = items[i]
        port.integrate_single(scenes.HALFSPACE, it["params"], it["rmin"], it["rmax"], it["method"], it["budget"],
                              it["seed"], nst_o)
        return evals_of(it)

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        cpu_evals = sum(ex.map(one, pick))
    batch_cpu_s = time.perf_counter() - t0
    out["batch"] = {
        "workload": "4096 independent integrals over [0,1]^d, d uniform in 2..6, prod_d exp(-a x)cos(b x) times a "
                    "random half-space indicator, budget log-uniform 256..65536 (MC samples or nested(simpson,"
                    "trapezoidal) regions), seed 11",
        "ms": round(ms, 2), "gsamples_s": round(runs[-1][0].evaluations / (ms * 1e6), 3),
        "evaluations": int(runs[-1][0].evaluations), "nested_regions": int(rep.nested_regions),
        "item_ms_p50": round(float(np.percentile(item_ms, 50)), 4),
        "item_ms_p99": round(float(np.percentile(item_ms, 99)), 2), "item_ms_max": round(float(item_ms.max()), 2),
        "threads": runs[-1][1].threads, "blocks": runs[-1][1].blocks,
        "e2e_ms": round(e2e_ms, 2),
        "timing": "resident: median of 3 graph launches (device); e2e: host items -> results through "
                  "vcu_integrate_batch, wall clock",
        "cpu_baseline": {"gsamples_s": round(cpu_evals / batch_cpu_s / 1e9, 4), "cores": threads, "kind": "port",
                         "sample": f"64 random items of at most 3 M evaluations ({cpu_evals} evaluations) in "
                                   f"{batch_cpu_s:.1f} s"}}
    out.update(adaptive_forms(ctx, port))
    out["learned_vs_plain"] = time_to_rmse(ctx)
    return out


def adaptive_forms(ctx, port) -> dict:
    """The other forms of the path, one line each: integrator_adaptive_iterations used directly (one
    heap over the range), the tolerance-driven form, and the control variates' importance strategies
    (rr_pdf_region + region_sampling_importance against the uniform choices, equal samples)."""
    from oracle import oracle as orc
    from viltrum_gb300 import _lib, scenes

    out = {}
    params = scenes.scene2(SEED)
    res = [512, 512]
    exact = scenes.exact_bins(scenes.SCENE2, params, [0, 0], [1, 1], res)
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], res)
    b = np.zeros(512 * 512, np.float32)
    # -- one heap of 2^18 regions over the whole range, accumulated into 512x512 bins
    st_abs = _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37)
    splits = (1 << 18) - 1

    def glob():
        b[:] = 0.0
        return ctx.adaptive_iterations_global(p, st_abs, splits, b)

    ms, st = _median_ms(glob, reps=3, warmup=3)
    t0 = time.perf_counter()
    port.adaptive_global(scenes.SCENE2, params, [0, 0], [1, 1], res, orc.Nested.make("simpson", "trapezoidal"), splits)
    cpu_s = time.perf_counter() - t0
    out["adaptive_global"] = {
        "workload": "integrator_adaptive_iterations(nested(simpson,trapezoidal), 2^18-1) used directly: one heap over "
                    "the 2-D scene, regions added into 512x512 bins",
        "ms": round(ms, 2), "regions": int(st.regions), "evaluations": int(st.evaluations),
        "rmse_vs_fp64": scenes.bin_rmse(b.reshape(-1, 1), exact), "timing": "median of 3 after 3 warm-up, device",
        "cpu_baseline": {"ms": round(cpu_s * 1e3, 1), "cores": 1, "kind": "port",
                         "sample": "the whole workload"}}
    # -- tolerance-driven: every region split until its error is below 1e-9
    bs_abs = _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)
    leaves = [0]

    def tol():
        b[:] = 0.0
        st_, n = ctx.adaptive_tolerance(p, bs_abs, 1e-9, b)
        leaves[0] = n
        return st_

    ms, st = _median_ms(tol, reps=3, warmup=3)
    t0 = time.perf_counter()
    _, cpu_leaves = port.adaptive_tolerance(scenes.SCENE2, params, [0, 0], [1, 1], res,
                                            orc.Nested.make("boole", "simpson"), 1e-9)
    cpu_s = time.perf_counter() - t0
    out["adaptive_tolerance"] = {
        "workload": "integrator_adaptive_tolerance(nested(boole,simpson), 1e-9) over the 2-D scene into 512x512 bins",
        "ms": round(ms, 2), "leaf_regions": int(leaves[0]), "evaluations": int(st.evaluations),
        "rmse_vs_fp64": scenes.bin_rmse(b.reshape(-1, 1), exact), "timing": "median of 3 after 3 warm-up, device",
        "cpu_baseline": {"ms": round(cpu_s * 1e3, 1), "cores": 1, "kind": "port", "leaf_regions": int(cpu_leaves),
                         "sample": "the whole workload"}}
    # -- the residual's region and point from the control variate's pdf, against the uniform ones
    res = [128, 128]
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], res)
    crespo = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
    b = np.empty(128 * 128, np.float32)
    lines = {}
    for name, rr, rs in (("uniform", 0, 0), ("rr_pdf_importance", 3, 1)):
        opts = _lib.CvOpts(16, 3, 1, 0, 0.0, rr, rs, 0.01, 0, 1.0, 0.0)
        ms, st = _median_ms(lambda: ctx.control_variates(p, crespo, (1 << 12) - 1, opts, b), reps=3, warmup=3)
        lines[name] = {"ms": round(ms, 3), "rmse_vs_fp64": scenes.bin_rmse(b.reshape(-1, 1), exact)}
    # -- crespo2021 with regions over (x, y) only, time integrated by Monte Carlo in every evaluation
    params = scenes.moving_scene3(SEED)
    res = [512, 512]
    p3 = ctx.problem(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res)
    b3 = np.empty(512 * 512 * 3, np.float32)
    fopts = _lib.CvOpts(64, 3, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 16)
    ms, st = _median_ms(lambda: ctx.control_variates(p3, crespo, (1 << 14) - 1, fopts, b3), reps=3, warmup=3)
    rows = list(range(0, 512, 64))
    err = np.concatenate([b3.reshape(512, 512, 3)[r] - scenes.exact_bins(
        scenes.MOVING_SCENE3, params, [0, r / 512.0, 0], [1, (r + 1) / 512.0, 1], [512, 1]) * 512.0 for r in rows])
    out["cv_fubini"] = {
        "workload": "integrator_crespo2021_infinite<2>(2^14-1 splits, 16 tail samples, 64 residual samples): regions "
                    "over x,y of the moving-disk scene (RGB, 512x512 bins), time by Monte Carlo in every evaluation",
        "ms": round(ms, 3), "gsamples_s": round(st.evaluations / (ms * 1e6), 3),
        "rmse_vs_fp64": float(np.sqrt(np.mean(err.astype(np.float64) ** 2))),
        "rmse_sample": f"{len(rows)} of 512 rows of bins", "timing": "median of 3 after 3 warm-up, device"}
    out["cv_importance"] = {
        "workload": "regions_integrator_parallel_variance_reduction(rr, cv_fixed_weight(0), sampler, 16 spp) over "
                    "2^12 regions of wave2, 128x128 bins: rr_uniform_region + region_sampling_uniform against "
                    "rr_pdf_region + region_sampling_importance",
        **lines, "timing": "median of 3 after 3 warm-up, device"}
    return out


def time_to_rmse(ctx, target: float = 1e-3, res_side: int = 1024, seeds=(1, 2, 3)) -> dict:
    """Time each estimator needs to reach bin RMSE <= target against the truth on the 5-D occluded
    scene (2 bin dims + 3 primary dims) at res_side^2 bins: plain Monte Carlo, the polynomial control
    variate (crespo2021, 2^14 regions) and the learned control variate (at most 12 000 Adam steps of
    32 768 samples, held-out checks every 200 with learning-rate drops on plateaus, the network's
    interpolant on 6 Simpson cells per primary dimension, per-bin weight from a pilot).  Per estimator and seed the samples per bin double until the target is met,
    starting from the power of two below the count a 256-sample run predicts; the time is the device
    time of the one call that met it (training and region construction included) and `spp_below`
    the largest count tried that did not.  The RMSE is taken over four 32x32 windows of the image
    (4096 bins), whose truth is plain Monte Carlo with 2^21 samples per bin (its squared standard
    error is subtracted).  A smaller closed-form case (sin(8x)e^-y + x^2 + y^2 at 8x8 bins) follows."""
    from viltrum_gb300 import _lib, scenes

    out = {}
    params = scenes.occluded_scene5(SEED)
    R = res_side
    p = ctx.problem(scenes.OCCLUDED_SCENE5, params, [0] * 5, [1] * 5, [R, R])
    nb = R * R
    W = 32
    corners = [(R // 8, R // 8), (R // 2, R // 4), (R // 4, 5 * R // 8), (3 * R // 4, 3 * R // 4)]
    idx, truth, se2 = [], [], []
    t0 = time.perf_counter()
    for cx, cy in corners:
        sub = ctx.problem(scenes.OCCLUDED_SCENE5, params, [cx / R, cy / R, 0, 0, 0],
                          [(cx + W) / R, (cy + W) / R, 1, 1, 1], [W, W])
        reps = []
        for k in range(2):
            b = np.empty(W * W, np.float32)
            ctx.per_bin_monte_carlo(sub, 1 << 20, 9000 + k, b)
            reps.append(b.astype(np.float64))
        # a window's bins are normalised by its own prod(res) = W^2: rescale to the image's R^2
        reps = np.array(reps) * (R * R) / (W * W)
        truth.append(reps.mean(axis=0))
        se2.append(reps.var(axis=0, ddof=1) / 2)
        jj, ii = np.meshgrid(np.arange(W), np.arange(W), indexing="ij")
        idx.append(((cy + jj) * R + (cx + ii)).ravel())
    idx = np.concatenate(idx)
    truth = np.concatenate(truth)
    se2 = float(np.mean(np.concatenate(se2)))
    truth_s = time.perf_counter() - t0

    def rmse(b):
        return float(np.sqrt(max(np.mean((b[idx].astype(np.float64) - truth) ** 2) - se2, 0.0)))

    buf = np.empty(nb, np.float32)

    def mc(spp, seed):
        st = ctx.per_bin_monte_carlo(p, spp, seed, buf)
        return st.device_ms, {}

    nst = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)

    def cv(spp, seed):
        st = ctx.control_variates(p, nst, (1 << 14) - 1, _lib.CvOpts(spp, seed, 0, 0, 1.0), buf)
        return st.device_ms, {}

    def lcv(spp, seed):
        st, rep = ctx.learned_control_variates(
            p, _lib.LearnedOpts(spp, seed, 12000, 32768, 3e-3, 200, 1, 0, None, 6), buf)
        return st.device_ms, {"train_steps": rep.train_steps_run, "train_ms": round(rep.train_ms, 2),
                              "grid_ms": round(rep.integral_ms, 2), "residual_ms": round(rep.residual_ms, 2),
                              "plain_mc_bins": rep.fallback_bins, "nodes_per_bin": rep.nodes_per_bin}

    def sweep(run, seed, cap):
        """smallest power-of-two samples per bin that reaches the target: start at the power of two
        below the count a 256-sample run predicts, halve while that still reaches, else double"""
        run(256, seed)
        need = 256 * (rmse(buf) / target) ** 2
        spp = 256
        while spp * 2 <= min(need, cap):
            spp *= 2
        tried = {}
        while 256 <= spp <= cap:
            ms, extra = run(spp, seed)
            e = rmse(buf)
            tried[spp] = (e <= target, e, ms, extra)
            if e <= target:
                if spp // 2 in tried or spp == 256:
                    break
                spp //= 2
            else:
                if spp * 2 in tried:
                    spp *= 2
                    break
                spp *= 2
        ok = [k for k, v in tried.items() if v[0]]
        if not ok:
            k = max(tried)
            return {"reached": False, "spp": k, "rmse": tried[k][1], "ms": round(tried[k][2], 2)}
        k = min(ok)
        below = [q for q, v in tried.items() if not v[0] and q < k]
        return {"reached": True, "spp": k, "spp_below": max(below) if below else None, "rmse": tried[k][1],
                "ms": round(tried[k][2], 2), **tried[k][3]}

    case = {"bins": [R, R], "rmse_bins": int(idx.size), "truth_spp": 2 << 20, "truth_s": round(truth_s, 1)}
    for name, run, cap in (("plain_mc", mc, 1 << 18), ("polynomial_cv", cv, 1 << 16), ("learned_cv", lcv, 1 << 17)):
        per = [sweep(run, seed, cap) for seed in seeds]
        reached = all(r["reached"] for r in per)
        case[name] = {"reached": reached, "mean_ms": round(float(np.mean([r["ms"] for r in per])), 2)
                      if reached else None, "seeds": per}
    m, l, c = case["plain_mc"], case["learned_cv"], case["polynomial_cv"]
    case["learned_over_plain_ms"] = round(l["mean_ms"] / m["mean_ms"], 3) if (m["reached"] and l["reached"]) else None
    case["learned_over_polynomial_ms"] = round(l["mean_ms"] / c["mean_ms"], 3) if (c["reached"] and l["reached"]) \
        else None
    out[f"occluded_scene5_{R}x{R}"] = case

    # the smooth 2-D case, closed-form truth, 8x8 bins
    p2 = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [8, 8])
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], [8, 8])[:, 0]
    b2 = np.empty(64, np.float32)

    def run2(kind, spp, seed):
        if kind == "plain_mc":
            return ctx.per_bin_monte_carlo(p2, spp, seed, b2).device_ms
        if kind == "polynomial_cv":
            return ctx.control_variates(p2, nst, (1 << 14) - 1, _lib.CvOpts(spp, seed, 0, 0, 1.0), b2).device_ms
        return ctx.learned_control_variates(p2, _lib.LearnedOpts(spp, seed, 4000, 32768, 3e-3, 200, 1, 4, None, 1),
                                            b2)[0].device_ms

    small = {}
    for kind in ("plain_mc", "polynomial_cv", "learned_cv"):
        per = []
        for seed in seeds:
            spp, res_ = 16, None
            while spp <= 1 << 20:
                ms = run2(kind, spp, seed)
                e = float(np.sqrt(np.mean((b2.astype(np.float64) - exact) ** 2)))
                if e <= target:
                    res_ = {"reached": True, "spp": spp, "rmse": e, "ms": round(ms, 3)}
                    break
                spp *= 2
            per.append(res_ or {"reached": False})
        ok = all(r["reached"] for r in per)
        small[kind] = {"reached": ok, "mean_ms": round(float(np.mean([r["ms"] for r in per])), 3) if ok else None,
                       "seeds": per}
    out["wave2_8x8"] = small
    out["target_rmse"] = target
    out["seeds"] = list(seeds)
    out["timing"] = "device time of the one call that reached the target (training and region construction " \
                    "included), mean over the seeds"
    return out


def _traffic_from_profile(nbins: int):
    """DRAM bytes per launch of the nested kernel: the per-bin figure of the committed ncu summary
    (captured on a 128x128 case) times this launch's bins (traffic grows with the bins written)."""
    path = os.path.join(ROOT, "profiles", "k_per_bin_nested_scene128.txt")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_bin:"):
                return round(float(ln.split(":")[1].split()[0]) * nbins)
    except OSError:
        pass
    return None


def cpu_baseline(args, sample_rows: int | None = None) -> dict:
    """The reference algorithm on the host cores (oracle restatement, bit-identical to the
    reference), over a bounded sample: the first `sample_rows` rows of bins."""
    from oracle import oracle as orc
    from viltrum_gb300 import scenes

    port = orc.port()
    params = scenes.scene2(SEED)
    threads = os.cpu_count() or 1
    rows = sample_rows or args.cpu_rows
    nbins = rows * RES[0]
    t0 = time.perf_counter()
    port.per_bin_adaptive_nested_threads(scenes.SCENE2, params, [0, 0], [1, 1], RES, orc.Nested.make(), ITERS, 0,
                                         nbins, threads)
    dt = time.perf_counter() - t0
    evals = nbins * (25 + ITERS * 20)
    return {"value": round(evals / dt / 1e9, 6), "unit": "Gsamples/s", "cores": threads, "kind": "port",
            "sample": f"first {rows} of {RES[1]} rows of bins ({nbins} bins, {evals} evaluations) in {dt:.2f} s"}


def run_reference(args) -> dict | None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    samples = []
    for _ in range(args.warmup):
        cpu_baseline(args, sample_rows=max(1, args.cpu_rows // 8))
    t_total = 0.0
    evals_total = 0
    for _ in range(args.steps):
        b = cpu_baseline(args)
        samples.append(b)
        nb = args.cpu_rows * RES[0]
        evals = nb * (25 + ITERS * 20)
        evals_total += evals
        t_total += evals / (b["value"] * 1e9)
    value = evals_total / t_total / 1e9
    base = samples[-1]
    return {
        "metric": METRIC, "value": round(value, 6), "unit": "Gsamples/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_total / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
        "data": "synthetic: 64 Gaussian bumps + 32 disks drawn by SplitMix64 (seed 7)",
        "config": {"workload": "per-bin adaptive nested Newton-Cotes: nested(boole,simpson), default absolute "
                               "heuristic, 15 splits (16 regions) per bin, 512x512 bins of the 2-D scene",
                   "bins": RES, "regions_per_bin": ITERS + 1,
                   "sample_per_step": f"first {args.cpu_rows} rows of bins",
                   "implementation": "the reference algorithm's CPU path restated in C++ (oracle/oracle.cc), "
                                     "bit-identical to the reference headers on the golden fixtures; "
                                     "bins split over all host threads"},
        "cpu_baseline": {"value": round(value, 6), "unit": "Gsamples/s", "cores": base["cores"], "kind": "port",
                         "sample": base["sample"]},
        "e2e": {"value": round(value, 6), "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def profile_workload(args) -> dict:
    """One small run of a single workload, for profiler captures (--workload): warm-up calls, then
    one call; prints its stats.  Not a benchmark line."""
    import torch

    import viltrum_gb300 as v
    from viltrum_gb300 import _lib, scenes

    torch.cuda.set_device(0)
    ctx = v.Context(0)
    r = args.res
    w = args.workload
    if w == "mc":
        p = ctx.problem(scenes.OCCLUDED_SCENE5, scenes.occluded_scene5(SEED), [0] * 5, [1] * 5, [r, r])
        b = np.empty(r * r, np.float32)
        call = lambda: ctx.per_bin_monte_carlo(p, 256, 5, b)
    elif w == "cv":
        p = ctx.problem(scenes.MOVING_SCENE3, scenes.moving_scene3(SEED), [0, 0, 0], [1, 1, 1], [r, r])
        b = np.empty(r * r * 3, np.float32)
        nst = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
        call = lambda: ctx.control_variates(p, nst, (1 << 12) - 1, _lib.CvOpts(16, 3, 0, 0, 1.0), b)
    elif w == "cv_crespo":  # the control-variate workload itself: crespo2021(2^14 - 1, 64), RGB moving scene
        p = ctx.problem(scenes.MOVING_SCENE3, scenes.moving_scene3(SEED), [0, 0, 0], [1, 1, 1], [r, r])
        b = np.empty(r * r * 3, np.float32)
        nst = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
        call = lambda: ctx.control_variates(p, nst, (1 << 14) - 1, _lib.CvOpts(64, 3, 0, 0, 1.0), b)
    elif w == "cv_occluded":  # the polynomial control variate of the time-to-RMSE sweep, 256 samples per bin
        p = ctx.problem(scenes.OCCLUDED_SCENE5, scenes.occluded_scene5(SEED), [0] * 5, [1] * 5, [r, r])
        b = np.empty(r * r, np.float32)
        nst = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
        call = lambda: ctx.control_variates(p, nst, (1 << 14) - 1, _lib.CvOpts(256, 1, 0, 0, 1.0), b)
    elif w in ("cv_importance", "cv_fubini"):
        nst = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
        if w == "cv_importance":  # rr_pdf_region + region_sampling_importance, alpha 0
            p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [r, r])
            b = np.empty(r * r, np.float32)
            opts = _lib.CvOpts(16, 3, 1, 0, 0.0, 3, 1, 0.01, 0, 1.0, 0.0)
        else:  # regions over (x, y), 16 tail samples of t per node value
            p = ctx.problem(scenes.MOVING_SCENE3, scenes.moving_scene3(SEED), [0, 0, 0], [1, 1, 1], [r, r])
            b = np.empty(r * r * 3, np.float32)
            opts = _lib.CvOpts(16, 3, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 16)
        call = lambda: ctx.control_variates(p, nst, (1 << 12) - 1, opts, b)
    elif w == "batch":
        items = _lib.batch_items(scenes.batch_items(256, seed=11, budget_hi=4096))
        nst = _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37)
        os.environ.setdefault("VCU_BATCH_THREADS", "512")
        call = lambda: ctx.integrate_batch(scenes.HALFSPACE, items, nst)[1]
    elif w == "learned":
        # the 5-D occluded scene with the options of the time-to-RMSE sweep (fewer training steps)
        p = ctx.problem(scenes.OCCLUDED_SCENE5, scenes.occluded_scene5(SEED), [0] * 5, [1] * 5, [r, r])
        b = np.empty(r * r, np.float32)
        opts = _lib.LearnedOpts(256, 5, 200, 32768, 3e-3, 0, 1, 0, None, 6)
        call = lambda: ctx.learned_control_variates(p, opts, b)[0]
    else:  # nested
        p = ctx.problem(scenes.SCENE2, scenes.scene2(SEED), [0, 0], [1, 1], [r, r])
        b = np.empty(r * r, np.float32)
        call = lambda: ctx.per_bin_adaptive_nested(p, _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37), ITERS, b)
    for _ in range(args.warmup):
        call()
    st = call()
    ctx.close()
    return {"workload": w, "res": r, "device_ms": st.device_ms, "evaluations": int(st.evaluations),
            "kernel_launches": int(st.kernel_launches)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-rows", type=int, default=64, help="rows of bins in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--res", type=int, default=512, help="bins per side (512 is the benchmark workload)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-configs", action="store_true", help="skip the other workloads' lines")
    ap.add_argument("--workload", choices=["nested", "mc", "cv", "cv_crespo", "cv_occluded", "cv_importance", "cv_fubini",
                             "batch", "learned"], default=None,
                    help="profiling aid: one small run of one workload (prints its stats, not a benchmark line)")
    args = ap.parse_args(argv)
    global RES
    RES = [args.res, args.res]
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.workload is not None:
        from viltrum_gb300 import build
        build.build()
        print(json.dumps(profile_workload(args)))
        return 0
    if args.impl == "reference":
        line = run_reference(args)
    else:
        from viltrum_gb300 import build
        build.build()
        line = run_ours(args)
    if line is not None:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
