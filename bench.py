"""Benchmark of the per-slide streaming DBSCAN path on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: 3-D random-walker stream (2,000 walkers, steps N(0, 1e-3)), window
W = 1,000,000, stride S = 10,000, Eps = 3.3328e-3 (mean neighbour count ~20),
MinPts = 10, FP64 neighbour relation (FP32 filter + FP64 band).  A step is one
slide.  Metric: slid points/s (S per slide).

value  -- device-resident: the whole stream sits in HBM before timing; each
          step is rtdbs_slide_async (D2D of the S new points into the engine,
          one CUDA-graph replay); CUDA events on the engine's stream around each
          step; L2 flushed (256 MB write) between steps outside the events.
e2e    -- through the host-buffer API with pinned buffers, every step the H2D
          of S points, the slide and the D2H of label[W] and cluster_id[W]:
          rtdbs_slide_pipelined (one slide in flight: each call returns the
          previous slide's result), host wall clock over all steps and the
          final sync -- the value; and rtdbs_slide (synchronous, L2 flushed
          before each call), host wall clock per call -- its latency.
With N > 1 (torchrun), every rank slides its own stream (seed + rank): the
path shards by stream with no collective (weak scaling).

Also on the line: the 2-D mixture stream with the reference's CPU path
timed and compared on every slide (W = 10,000, 100 slides), the precision
stream (W = 500,000, FP64 band re-checks, mismatches against the FP64
oracle), 256 uneven streams batched in a pool, and the continuous-batching
server over 1,000 streams (with and without a binding HBM budget).

--impl reference: the reference's CPU path (cluster_with_cpu,
src/dbscan/util.cpp:299-354, through the oracle's restatement; the
reference's own build cannot run on the GPU machine) on every host core.  It is
O(W^2) per slide, so on the walker stream a step is a bounded sample -- one
16,384-point window of the same walker density per host thread -- and the
slid points/s at W = 1M are projected by (W/16384)^2; the 2-D mixture stream
is measured in full.
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

from rtdbstream_gb300 import workloads as wl  # noqa: E402

METRIC = "slid points/s"
UNIT = "points/s"
SPEC = wl.CFG1
WORKLOAD = "walkers3d W=1,000,000 S=10,000 Eps=3.3328e-3 MinPts=10 fp64"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--profile-steps", type=int, default=5)
    ap.add_argument("--no-verify", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-extra-configs", action="store_true")
    # smaller windows of the same walker stream, for profiler captures only
    ap.add_argument("--window", type=int, default=None)
    ap.add_argument("--stride", type=int, default=None)
    args = ap.parse_args()
    global SPEC, WORKLOAD
    if args.window or args.stride:
        W = args.window or SPEC.window
        S = args.stride or SPEC.stride
        SPEC = wl.StreamSpec(f"walkers3d-W{W}-S{S}", 3, W, S, SPEC.eps, SPEC.min_pts, SPEC.slides)
        WORKLOAD = f"walkers3d W={W:,} S={S:,} Eps={SPEC.eps} MinPts={SPEC.min_pts} fp64"
    return args


def weak_scaling_value(local_ms: float, steps: int, stride: int, world: int, device: str = "cpu"):
    """Whole-job slid points/s of `world` independent streams, one per rank:
    every rank slid steps * stride points; the job time is the slowest rank's
    (MAX over ranks).  Returns (value, max_ms)."""
    total_ms = local_ms
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([local_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
        total_ms = float(t.item())
    return world * steps * stride / (total_ms / 1000.0), total_ms


def walker_stream(n_total: int, seed: int, window: int = None) -> np.ndarray:
    """The walker stream; a smaller window keeps 500 points per walker trail
    (2,000 walkers at W = 1M), so the local density matches the full size."""
    walkers = max(1, round(2000 * (window or SPEC.window) / 1_000_000))
    return wl.random_walkers(n_total, n_walkers=walkers, seed=seed)


def partition_streams(costs, world: int, rank: int) -> list:
    """Indices of the streams rank `rank` of `world` serves: streams are
    independent, so the pool and the server shard by stream with no
    collective; greedy longest-first by cost keeps the ranks' work even."""
    load = [0.0] * world
    owner = [0] * len(costs)
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(costs)) if owner[i] == rank]


def combine_ranks(points: float, ms: float, world: int, device: str = "cpu"):
    """Whole-job slid points/s of sharded work: points summed over ranks,
    time = the slowest rank's.  Returns (value, total_points, max_ms)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([points], dtype=torch.float64, device=device)
        m = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        points, ms = float(t.item()), float(m.item())
    return points / (ms / 1000.0), points, ms


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ------------------------------------------------------------ CPU reference

SUB = 16_384  # points of one sampled window of the reference's O(W^2) path


def host_threads() -> int:
    return os.cpu_count() or 1


def cpu_reference_steps(steps: int, threads: int, seed: int = 11) -> dict:
    """The reference's CPU path (restated cluster_with_cpu, FP32, O(W^2)) on
    the walker stream: each step clusters one 16,384-point window per host
    thread, in parallel (windows of a walker stream with 33 walkers, so the
    trails have the density of the 1M window); the slid points/s at the full
    window are projected by the W^2 cost law of both of its loops."""
    import concurrent.futures as cf

    import oracle

    oracle.build(ref=False)
    S_sub = max(1, SUB // 100)
    pts = walker_stream(SUB + 64 * S_sub, seed=seed, window=SUB)

    def one(k):
        win = oracle.window_of(pts, SUB, S_sub, k % 64)
        t0 = time.perf_counter()
        oracle.window_bruteforce(win, SPEC.eps, SPEC.min_pts)
        return time.perf_counter() - t0

    per, walls = [], []
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for s in range(steps):
            t0 = time.perf_counter()
            per.extend(ex.map(one, range(s * threads, (s + 1) * threads)))
            walls.append(time.perf_counter() - t0)
    mean_sample = statistics.mean(per)
    scale = (SPEC.window / SUB) ** 2
    value = threads * SPEC.stride / (mean_sample * scale)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "value_kind": "projected",
            "ms_per_step": 1000.0 * statistics.mean(walls),
            "sample": (f"restated cluster_with_cpu on {len(per)} windows of {SUB} points of a walker stream of the "
                       f"same trail density ({steps} step(s) of {threads} window(s) in parallel, mean "
                       f"{mean_sample:.3f} s per window on one thread), projected to W={SPEC.window} by "
                       f"(W/{SUB})^2")}


def cpu_cfg0(threads: int, seed: int = 0, slides: int = None):
    """The reference's CPU path (restated cluster_with_cpu) on every slide
    of the 2-D mixture stream (W = 10,000, S = 1,000, Eps 0.5, MinPts 5),
    measured in full: returns ({slide: (nn, label, cid)}, summary)."""
    import concurrent.futures as cf

    import oracle

    oracle.build(ref=False)
    sp = wl.CFG0
    n = slides or sp.slides
    pts = wl.cfg0_stream(seed=seed)

    def one(k):
        win = oracle.window_of(pts, sp.window, sp.stride, k)
        t0 = time.perf_counter()
        out = oracle.window_bruteforce(win, sp.eps, sp.min_pts)
        return k, out, time.perf_counter() - t0

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, range(1, n + 1)))
    wall = time.perf_counter() - t0
    per = [r[2] for r in res]
    summary = {"slides": n, "cores": threads, "kind": "port", "wall_s": wall,
               "slid_points_per_s": n * sp.stride / wall,
               "ms_per_slide_one_thread_mean": 1000.0 * statistics.mean(per),
               "sample": f"restated cluster_with_cpu on all {n} slides, {threads} slide(s) at a time"}
    return {k: out for k, out, _ in res}, summary


def run_reference(args) -> None:
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = host_threads()
    steps = max(1, args.steps)
    base = cpu_reference_steps(steps, threads)
    _, cfg0 = cpu_cfg0(threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": base["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_block(),
        "value_kind": "projected",
        "step": (f"{threads} windows of {SUB} points clustered in parallel, a bounded sample of one W = "
                 f"{SPEC.window:,} slide; value = slid points/s at W = {SPEC.window:,} projected by the W^2 law"),
        "cpu_baseline": base,
        "cfg0_measured": cfg0,
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- our engine

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, interval_ms: int = 20):
        self.gpu = gpu_index
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the sampler is live (its first sample is in) before the timed work starts
            t_end = time.time() + 5.0
            while not self.lines and self.proc.poll() is None and time.time() < t_end:
                time.sleep(0.005)
            self.lines.clear()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(phase: str, W: int, S: int, dim: int, cells: int, items: int) -> float:
    """Compulsory DRAM bytes of one launch of a phase (each live structure
    touched once; neighbour candidates re-read from cache are not counted)."""
    c = min(S, 16384)
    return {
        "ingest": c * (4 * dim + 16 + 8 + 16 + 8 + 8 + 8 + 16),
        "sort": 2 * c * 16,
        "decrement": c * (8 + 16),
        # (key, point, count) read and written, root hint written, the previous
        # root carried (read and written) while forest reuse is on
        "merge": W * (28 + 28 + 4 + 8) + c * (8 + 16),
        "build": W * 8 + cells * 32 + items * 8,
        "increment": c * (8 + 16) + c * 4,
        "union": W * (16 + 4 + 4 + 4),
        # scnt, slot, root hint, parent read; root by slot and by position written
        "flatten": W * (4 + 4 + 4 + 4 + 4 + 4),
        # border pass: root by slot read; label, cid, parent, damage mark written
        "label": W * (4 + 4 + 4 + 4 + 4),
    }[phase]


def config_block() -> dict:
    """The workload both arms report (identical keys and values)."""
    return {"workload": WORKLOAD, "window": SPEC.window, "stride": SPEC.stride, "eps": SPEC.eps,
            "min_pts": SPEC.min_pts, "dim": 3, "precision": "fp64 neighbour relation (fp32 filter + fp64 band)",
            "l2": "flushed between steps (256 MB write outside the timed events)",
            "parallelism": "one independent stream per GPU (weak scaling)"}


# CUDA-core FP32 peak, nominal: 152 SMs x 128 FP32 lanes x 2 (an FMA, or a
# paired f32x2 operation, per lane and cycle) x 2.07 GHz.  The measured-peaks
# file holds no CUDA-core figure.
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def fp32_ops_per_test(dim: int) -> int:
    """FP32 operations of one distance test: dim differences, dim squares,
    dim - 1 sums and the comparison."""
    return 3 * dim + 1


def measured_peak() -> tuple:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(phase: str):
    """DRAM bytes per launch of the dominant kernel at W = 1M from the
    committed ncu summary (profiles/ncu_traffic.json, captured at the
    bench's own size), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get({"label": "k_border"}.get(phase, f"k_{phase}"))
    except (OSError, ValueError):
        return None


def headline_summary(line: dict) -> dict:
    """The line's headline figures, rounded, in a few hundred characters:
    printed as the line's last key so that a reader keeping only the end of
    the output still has them (the full blocks stay above)."""
    def r(x, n=3):
        return None if x is None else float(f"{x:.{n}g}")

    out = {"walker": {"ms_per_slide": r(line.get("ms_per_step"), 4), "value": r(line.get("value")),
                      "e2e_pipelined": r((line.get("e2e") or {}).get("value")),
                      "e2e_synchronous": r(((line.get("e2e") or {}).get("synchronous") or {}).get("value")),
                      "exact_vs_fp64_oracle": line.get("exact_vs_fp64_oracle"),
                      "union_roofline_frac": r((line.get("roofline") or {}).get("frac"))}}
    c0 = line.get("cfg0")
    if c0:
        out["cfg0"] = {"value": r(c0["value"]), "e2e": r(c0["e2e"]["value"]),
                       "e2e_pipelined": r(c0["e2e_pipelined"]["value"]),
                       "slides_exact_vs_reference_cpu": c0["slides_exact_vs_reference_cpu"],
                       "cpu_reference": r(c0["cpu_reference"]["slid_points_per_s"])}
    c2 = line.get("cfg2")
    if c2:
        out["cfg2"] = {"value": r(c2["value"]), "rechecked_pairs_per_slide": c2["rechecked_pairs_per_slide"],
                       "mismatches_vs_fp64_oracle": c2["mismatches_vs_fp64_oracle"]}
    b = line.get("batched")
    if b:
        out["batched"] = {"value": r(b["value"]), "round_ms_p50": r(b["round_ms_p50"]),
                          "speedup_vs_tuned_plain": r(b["speedup_vs_plain"]),
                          "speedup_vs_fixed_plain": r(b["value"] / b["plain_one_at_a_time_default"]["value"]),
                          "streams_exact_vs_fp64_oracle": b["streams_exact_vs_fp64_oracle"]}
    sv = line.get("serving")
    if sv:
        out["serving"] = {"capacity_requests_per_s": r(sv["capacity_requests_per_s"]),
                          "p50_p99_ms_by_load": {str(e["offered_fraction"]): [r(e["latency_ms_p50"]),
                                                                               r(e["latency_ms_p99"])]
                                                 for e in sv["sweep"]}}
    return out


def run_ours(args) -> None:
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    from rtdbstream_gb300 import Engine

    W, S = SPEC.window, SPEC.stride
    total_steps = args.warmup + args.steps + 2 * args.e2e_steps + args.profile_steps
    pts = walker_stream(W + total_steps * S, seed=1 + rank)
    d_pts = torch.from_numpy(pts).to(f"cuda:{dev}")
    # One dedicated stream for the engine, the timing events and the L2 flush
    # (torch's default stream is the legacy NULL stream, which the engine
    # would replace by a private stream of its own).
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    eng = Engine(3, W, S, SPEC.eps, SPEC.min_pts, precision="fp64", device=dev,
                 stream=stream.cuda_stream)
    eng.load_window(pts[:W])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    step = 0

    def new_pts(k):
        return d_pts[W + k * S: W + (k + 1) * S]

    for _ in range(args.warmup):
        eng.slide_async(new_pts(step))
        step += 1
    eng.sync()
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # clocks sampled over the timed loops (device-resident, then end to end)
    clk = ClockSampler(dev).__enter__()
    for k in range(args.steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        eng.slide_async(new_pts(step))
        ends[k].record(stream)
        step += 1
    eng.sync()
    torch.cuda.synchronize()
    per_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    value, total_ms = weak_scaling_value(float(sum(per_ms)), args.steps, S, world, f"cuda:{dev}")

    # end to end through the host-buffer API (pinned buffers)
    h_pts = torch.from_numpy(pts).pin_memory().numpy()
    h_lab = torch.empty(W, dtype=torch.int32).pin_memory().numpy()
    h_cid = torch.empty(W, dtype=torch.int32).pin_memory().numpy()
    e2e_s = []
    for _ in range(args.e2e_steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.slide(h_pts[W + step * S: W + (step + 1) * S], h_lab, h_cid)
        e2e_s.append(time.perf_counter() - t0)
        step += 1
    e2e_sync_value = S / statistics.mean(e2e_s) if e2e_s else None
    # pipelined: one slide in flight, outputs alternate between two pinned
    # buffer pairs (a pair is free again once the call after next returns);
    # the engine's ~220 MB working set per slide exceeds L2, so no flush
    outs = [(torch.empty(W, dtype=torch.int32).pin_memory().numpy(),
             torch.empty(W, dtype=torch.int32).pin_memory().numpy()) for _ in range(2)]
    e2e_value = None
    if args.e2e_steps:
        eng.sync()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.e2e_steps):
            eng.slide_pipelined(h_pts[W + step * S: W + (step + 1) * S], *outs[k % 2])
            step += 1
        eng.sync()
        e2e_value = S * args.e2e_steps / (time.perf_counter() - t0)
    clk.__exit__(None, None, None)

    # per-phase device times (direct launches bracketed by events) and the
    # counters of the same slides
    prof = []
    st0 = eng.stats()
    for _ in range(args.profile_steps):
        flush.fill_(2.0)
        prof.append(eng.slide_profiled(new_pts(step)))
        step += 1
    st = eng.stats()
    nprof = max(1, st["slides"] - st0["slides"])
    per_slide = {k: (st[k] - st0[k]) / nprof for k in ("query_tests", "query_hits", "cluster_tests",
                                                        "cluster_hits", "band_rechecks")}
    phases = ["ingest", "sort", "decrement", "merge", "build", "increment", "union", "flatten", "label"]
    avg = {p: statistics.mean(x[f"{p}_ms"] for x in prof) for p in phases} if prof else {}
    verified = None
    if rank == 0 and not args.no_verify:
        import oracle

        oracle.build(ref=False)
        win = oracle.window_of(pts, W, S, step)
        exp_nn, exp_lab, exp_cid, _ = oracle.window_grid(win, SPEC.eps, SPEC.min_pts, oracle.MODE_FP64)
        lab, cid = eng.cluster()
        verified = bool(np.array_equal(lab, exp_lab) and np.array_equal(cid, exp_cid)
                        and np.array_equal(eng.counts(), exp_nn))
    eng.close()
    del d_pts

    peak, peak_kind = measured_peak()
    roofline = None
    if rank == 0 and avg:
        roofline = roofline_block(avg, st, per_slide, W, S, total_ms / args.steps, peak, peak_kind)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_reference_steps(2, host_threads())
        cpu.pop("ms_per_step", None)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_block(),
        "latency_ms": {"p50": float(np.percentile(per_ms, 50)), "p99": float(np.percentile(per_ms, 99))},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": S * 3 * 4,
                "d2h_bytes_per_step": 2 * W * 4,
                "api": "rtdbs_slide_pipelined, pinned host buffers, one slide in flight",
                "synchronous": {"api": "rtdbs_slide", "value": e2e_sync_value,
                                "latency_ms_p50": 1000 * float(np.percentile(e2e_s, 50)) if e2e_s else None}},
        "gpu_launches": args.steps * st["launches_per_slide"],
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "exact_vs_fp64_oracle": verified,
        "counters_per_slide": {**{k: round(v) for k, v in per_slide.items()},
                               "max_query_tests": st["max_query_tests"], "reused_cores": st["reused_cores"]},
    }
    if not args.no_extra_configs:
        if rank == 0:
            line["cfg0"] = run_cfg0(args, dev, stream)
            line["cfg2"] = run_cfg2(args, dev, stream, flush)
        if world > 1:
            torch.distributed.barrier()
    if not args.no_batched:
        line["batched"] = run_batched(args, dev, stream, flush, world, rank)
    if not args.no_serving:
        line["serving"] = run_serving(args, dev, stream, world, rank)
    if rank == 0:
        try:
            line["summary"] = headline_summary(line)  # last: the line's tail carries the headline figures
        except (KeyError, TypeError, ValueError) as e:  # a missing figure must not cost the line
            print(f"bench: no summary ({e!r})", file=sys.stderr)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def roofline_block(avg, st, per_slide, W, S, slide_ms, peak, peak_kind) -> dict:
    """Slower-of roofline of the dominant kernel: algorithmic bytes / HBM
    peak against algorithmic FP32 operations / CUDA-core FP32 peak (the
    distance tests the kernel evaluates, 3d + 1 operations each)."""
    phases = list(avg)
    dom = max(avg, key=avg.get)
    launches = st["chunks_per_slide"] if dom not in ("union", "flatten", "label") else 1
    alg = algorithmic_bytes(dom, W, S, 3, st["cells"], st["work_items"]) * launches
    tests = {"union": per_slide["cluster_tests"], "decrement": per_slide["query_tests"] / 2,
             "increment": per_slide["query_tests"] / 2}.get(dom, 0.0)
    flops = fp32_ops_per_test(3) * tests
    t_bytes = alg / (peak * 1e9)
    t_flops = flops / (FP32_PEAK_TFLOPS * 1e12)
    t = avg[dom] / 1000.0
    achieved = alg / t / 1e9
    slide_alg = sum(algorithmic_bytes(p, W, S, 3, st["cells"], st["work_items"]) for p in phases)
    return {"bound": "hbm" if t_bytes >= t_flops else "fp32", "kernel": dom, "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
            "traffic": ncu_traffic(dom), "algorithmic_bytes_per_launch": alg,
            "fp32": {"ops_per_launch": flops, "achieved_tflops": flops / t / 1e12,
                     "peak_tflops": FP32_PEAK_TFLOPS, "peak_source": "nominal CUDA-core FP32",
                     "frac": flops / t / 1e12 / FP32_PEAK_TFLOPS},
            "terms_us": {"bytes_over_hbm": 1e6 * t_bytes, "fp32_over_cuda_cores": 1e6 * t_flops,
                         "measured": 1e6 * t},
            "slower_of_frac": max(t_bytes, t_flops) / t,
            "phase_ms": avg,
            "slide": {"algorithmic_bytes": slide_alg,
                      "achieved_gbs": slide_alg / (slide_ms / 1000.0) / 1e9,
                      "frac": slide_alg / (slide_ms / 1000.0) / 1e9 / peak}}


def run_cfg0(args, dev, stream) -> dict:
    """2-D Gaussian mixture (W = 10,000, S = 1,000, 100 slides, Eps 0.5,
    MinPts 5) in the reference's FP32 predicate: every slide's counts, labels
    and ids compared with the reference's CPU path, which is timed on every
    slide.  Device-resident slides timed with CUDA events, then the same
    stream end to end through rtdbs_slide with host buffers, and through
    rtdbs_slide_pipelined (one slide in flight)."""
    import torch

    from rtdbstream_gb300 import Engine

    sp = wl.CFG0
    pts = wl.cfg0_stream(seed=0)
    ref, cpu = cpu_cfg0(host_threads())
    d = torch.from_numpy(pts).to(f"cuda:{dev}")

    def win(k):
        return d[sp.window + k * sp.stride: sp.window + (k + 1) * sp.stride]

    eng = Engine(2, sp.window, sp.stride, sp.eps, sp.min_pts, precision="fp32", device=dev,
                 stream=stream.cuda_stream)
    eng.load_window(pts[:sp.window])
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(sp.slides)]
    for k, (a, b) in enumerate(ev):
        a.record(stream)
        eng.slide_async(win(k))
        b.record(stream)
    eng.sync()
    torch.cuda.synchronize()
    per_ms = [a.elapsed_time(b) for a, b in ev]
    eng.close()
    # end to end, and exactness on every slide against the reference's CPU path
    eng = Engine(2, sp.window, sp.stride, sp.eps, sp.min_pts, precision="fp32", device=dev,
                 stream=stream.cuda_stream)
    eng.load_window(pts[:sp.window])
    h_lab = torch.empty(sp.window, dtype=torch.int32).pin_memory().numpy()
    h_cid = torch.empty(sp.window, dtype=torch.int32).pin_memory().numpy()
    e2e_s, bad = [], []
    for k in range(sp.slides):
        new = pts[sp.window + k * sp.stride: sp.window + (k + 1) * sp.stride]
        t0 = time.perf_counter()
        eng.slide(new, h_lab, h_cid)
        e2e_s.append(time.perf_counter() - t0)
        enn, elab, ecid = ref[k + 1]
        if not (np.array_equal(h_lab, elab) and np.array_equal(h_cid, ecid) and np.array_equal(eng.counts(), enn)):
            bad.append(k + 1)
    eng.close()
    # end to end with one slide in flight (rtdbs_slide_pipelined): pinned input
    # stride, two pinned output sets used in turn; host wall clock over all
    # slides and the final sync; the last slide's outputs checked
    eng = Engine(2, sp.window, sp.stride, sp.eps, sp.min_pts, precision="fp32", device=dev,
                 stream=stream.cuda_stream)
    eng.load_window(pts[:sp.window])
    p_pts = torch.from_numpy(pts).pin_memory().numpy()
    outs = [tuple(torch.empty(sp.window, dtype=torch.int32).pin_memory().numpy() for _ in range(2))
            for _ in range(2)]
    t0 = time.perf_counter()
    for k in range(sp.slides):
        eng.slide_pipelined(p_pts[sp.window + k * sp.stride: sp.window + (k + 1) * sp.stride], *outs[k % 2])
    eng.sync()
    pipe_s = time.perf_counter() - t0
    _, elab, ecid = ref[sp.slides]
    last_lab, last_cid = outs[(sp.slides - 1) % 2]
    pipe_exact = bool(np.array_equal(last_lab, elab) and np.array_equal(last_cid, ecid))
    eng.close()
    gpu_value = sp.slides * sp.stride / (sum(per_ms) / 1000.0)
    return {"workload": f"2-D mixture W={sp.window:,} S={sp.stride:,} Eps={sp.eps} MinPts={sp.min_pts}, "
                        f"{sp.slides} slides, fp32 (the reference's predicate)",
            "value": gpu_value, "unit": UNIT,
            "latency_ms": {"p50": float(np.percentile(per_ms, 50)), "p99": float(np.percentile(per_ms, 99))},
            "e2e": {"value": sp.slides * sp.stride / sum(e2e_s), "unit": UNIT,
                    "latency_ms_p50": 1000 * float(np.percentile(e2e_s, 50)),
                    "latency_ms_p99": 1000 * float(np.percentile(e2e_s, 99))},
            "e2e_pipelined": {"value": sp.slides * sp.stride / pipe_s, "unit": UNIT,
                              "api": "rtdbs_slide_pipelined, pinned host buffers, one slide in flight",
                              "last_slide_exact": pipe_exact},
            "cpu_reference": cpu,
            "e2e_vs_cpu_reference": sp.slides * sp.stride / sum(e2e_s) / cpu["slid_points_per_s"],
            "slides_exact_vs_reference_cpu": sp.slides - len(bad), "slides_differing": bad}


def run_cfg2(args, dev, stream, flush, slides: int = 20, checked: int = 3) -> dict:
    """Precision stream (W = 500,000, S = 5,000, Eps 1e-3, MinPts 8;
    coordinates with a large common offset and 5% of the points at
    Eps (1 +- 1e-6) from a partner): slid points/s in the FP64 relation,
    pair tests re-decided in FP64 per slide, and the last `checked` slides'
    own outputs compared with the FP64 oracle (mismatches must be 0); also
    how many labels the reference's FP32 predicate would get wrong there."""
    import torch

    import oracle
    from rtdbstream_gb300 import Engine

    sp = wl.CFG2
    W, S = sp.window, sp.stride
    warm = 3
    pts = wl.cfg2_stream(n_total=W + (warm + slides) * S)
    d = torch.from_numpy(pts).to(f"cuda:{dev}")
    eng = Engine(3, W, S, sp.eps, sp.min_pts, precision="fp64", device=dev, stream=stream.cuda_stream)
    eng.load_window(pts[:W])
    for k in range(warm):
        eng.slide_async(d[W + k * S: W + (k + 1) * S])
    eng.sync()
    st0 = eng.stats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(slides)]
    d_lab = torch.empty(W, dtype=torch.int32, device=f"cuda:{dev}")
    d_cid = torch.empty(W, dtype=torch.int32, device=f"cuda:{dev}")
    mism = {"counts": 0, "labels": 0, "ids": 0}
    fp32_wrong = 0
    for i, (a, b) in enumerate(ev):
        k = warm + i
        check = i >= slides - checked
        flush.fill_(float(k))
        a.record(stream)
        if check:  # this slide's own outputs (one 4 MB device copy each)
            eng.slide_async(d[W + k * S: W + (k + 1) * S], d_lab, d_cid)
        else:
            eng.slide_async(d[W + k * S: W + (k + 1) * S])
        b.record(stream)
        if check:
            torch.cuda.synchronize()
            win = oracle.window_of(pts, W, S, k + 1)
            enn, elab, ecid, _ = oracle.window_grid(win, sp.eps, sp.min_pts, oracle.MODE_FP64)
            lab, cid = d_lab.cpu().numpy(), d_cid.cpu().numpy()
            mism["counts"] += int(np.sum(eng.counts() != enn))
            mism["labels"] += int(np.sum(lab != elab))
            mism["ids"] += int(np.sum(cid != ecid))
            _, flab, _, _ = oracle.window_grid(win, sp.eps, sp.min_pts, oracle.MODE_FP32)
            fp32_wrong += int(np.sum(flab != elab))
    eng.sync()
    torch.cuda.synchronize()
    st = eng.stats()
    eng.close()
    per_ms = [a.elapsed_time(b) for a, b in ev]
    n = st["slides"] - st0["slides"]
    return {"workload": f"offset 3-D W={W:,} S={S:,} Eps={sp.eps} MinPts={sp.min_pts}, 5% of points at "
                        f"Eps(1 +- 1e-6), fp64 relation (fp32 filter + fp64 band), {slides} timed slides",
            "value": slides * S / (sum(per_ms) / 1000.0), "unit": UNIT,
            "latency_ms": {"p50": float(np.percentile(per_ms, 50)), "p99": float(np.percentile(per_ms, 99))},
            "rechecked_pairs_per_slide": (st["band_rechecks"] - st0["band_rechecks"]) / max(1, n),
            "dist_tests_per_slide": (st["dist_tests"] - st0["dist_tests"]) / max(1, n),
            "checked_slides": checked, "mismatches_vs_fp64_oracle": mism,
            "labels_the_fp32_predicate_gets_wrong": fp32_wrong}


def exact_vs_oracle(pairs, threads: int) -> list:
    """Indices of the (window, spec, label, cid) entries whose result
    differs from the FP64 oracle (checked on the host cores in parallel)."""
    import concurrent.futures as cf

    import oracle

    oracle.build(ref=False)

    def one(i):
        win, st, lab, cid = pairs[i]
        _, elab, ecid, _ = oracle.window_grid(win, st.eps, st.min_pts, oracle.MODE_FP64)
        return i if not (np.array_equal(lab, elab) and np.array_equal(cid, ecid)) else None

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return [i for i in ex.map(one, range(len(pairs))) if i is not None]


def run_batched(args, dev, stream, flush, world=1, rank=0, n_streams=256, rounds=None, plain_rounds=4):
    """256 uneven streams slid together by a pool (one launch per phase, a
    CUDA-graph replay per round) against the same streams slid one at a time
    by single-stream engines.  Device-resident inputs, CUDA events per round,
    L2 flushed between rounds outside the events.  With N ranks each serves
    its share of the streams (no collective on the data path); the whole-job
    rate is all ranks' slid points over the slowest rank's time."""
    import torch

    from rtdbstream_gb300 import Engine, Pool, make_params

    all_streams = wl.mixed_streams(n_streams)
    mine = partition_streams([st.window for st in all_streams], world, rank)
    streams = [wl.calibrate_eps(all_streams[i]) for i in mine]  # Eps fitted per stream
    n_streams = len(streams)
    rounds = rounds or (args.warmup + max(10, args.steps // 5))
    data = [wl.mix_points(st, st.window + rounds * st.stride) for st in streams]
    # launch configuration (cells per Eps, work split) per stream bucket, picked
    # by the autotuner on each bucket's first stream; pool and plain engines use it
    from rtdbstream_gb300.autotune import Autotuner

    # (pool rounds for the pool, single engines for the plain path: each at its best)
    tuner = Autotuner(cache_path=os.path.join(ROOT, "_build", "autotune_batched.json"), device=dev)
    tuned = tuner.choose_batched([(d, st.dim, st.window, st.stride, st.eps, st.min_pts, "fp64")
                                  for st, d in zip(streams, data)])
    tuned_plain = [tuner.choose(d, st.dim, st.window, st.stride, st.eps, st.min_pts) for st, d in zip(streams, data)]
    packed = [torch.from_numpy(np.concatenate([d[st.window + k * st.stride: st.window + (k + 1) * st.stride]
                                               .reshape(-1) for st, d in zip(streams, data)])).to(dev)
              for k in range(rounds)]
    pool = Pool(device=dev, use_graph=True, stream=stream.cuda_stream)
    ids = []
    for st, d in zip(streams, data):
        c = tuned[len(ids)]
        sid = pool.add_stream(make_params(st.dim, st.window, st.stride, st.eps, st.min_pts, device=dev,
                                          cell_mult=c["cell_mult"], work_grab=c["work_grab"],
                                          query_lanes=c["query_lanes"]))
        pool.load_window(sid, d[:st.window])
        ids.append(sid)
    # the mean neighbour count (self included) each stream's Eps gives, from
    # the engine's exact counts of its first window
    mean_nn = np.array([float(pool.counts(sid).mean()) for sid in ids])
    for k in range(args.warmup):
        pool.slide(ids, packed[k])
    pool.sync()
    timed = list(range(args.warmup, rounds))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in timed]
    for (a, b), k in zip(ev, timed):
        flush.fill_(float(k))
        a.record(stream)
        pool.slide(ids, packed[k])
        b.record(stream)
    pool.sync()
    per_round = [a.elapsed_time(b) for a, b in ev]
    slid = sum(st.stride for st in streams)
    value, _, _ = combine_ranks(slid * len(timed), sum(per_round), world, f"cuda:{dev}")
    # exactness of every stream against the FP64 oracle
    import oracle

    pairs = [(oracle.window_of(data[i], st.window, st.stride, rounds), st) + tuple(pool.outputs(ids[i]))
             for i, st in enumerate(streams)]
    differing = exact_vs_oracle(pairs, host_threads())
    del pairs
    # one more round (the last round's points again) with every phase timed
    prof = pool.slide_profiled(ids, packed[timed[-1]])
    prof = {k: v for k, v in prof.items() if k.endswith("_ms")}
    stats = pool.stats()
    pool.close()

    # the plain path: the same streams, one engine each, slid one at a time
    # (with the autotuner's single-engine choices, and with the default
    # configuration for reference)
    offsets, o = [], 0
    for st in streams:
        offsets.append(o)
        o += st.stride * st.dim

    def plain_round_ms(configs):
        engines = []
        for st, d, c in zip(streams, data, configs):
            e = Engine(st.dim, st.window, st.stride, st.eps, st.min_pts, device=dev, stream=stream.cuda_stream,
                       cell_mult=c["cell_mult"], work_grab=c["work_grab"], query_lanes=c["query_lanes"])
            e.load_window(d[:st.window])
            engines.append(e)
        ms = []
        for k in range(min(plain_rounds, rounds)):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for e, st, off in zip(engines, streams, offsets):
                e.slide_async(packed[k][off: off + st.stride * st.dim])
            b.record(stream)
            torch.cuda.synchronize()
            if k > 0:
                ms.append(a.elapsed_time(b))
        for e in engines:
            e.close()
        return statistics.mean(ms)

    plain_ms = plain_round_ms(tuned_plain)
    default_ms = plain_round_ms([{"cell_mult": 1, "work_grab": 8, "query_lanes": 16}] * len(streams))
    plain_value, _, _ = combine_ranks(slid, plain_ms, world, f"cuda:{dev}")
    default_value, _, _ = combine_ranks(slid, default_ms, world, f"cuda:{dev}")
    # the tuner's per-bucket choices go to a file beside its cache, not on the line
    choices_file = os.path.join(ROOT, "_build", "bench_autotune_choices.json")
    if rank == 0:
        os.makedirs(os.path.dirname(choices_file), exist_ok=True)
        with open(choices_file, "w") as f:
            json.dump({k: [v["cell_mult"], v["work_grab"], v.get("query_lanes")]
                       for k, v in sorted(tuner.cache.items())}, f, indent=1)
    n_diff, _, _ = combine_ranks(len(differing), 1000.0, world, f"cuda:{dev}")
    return {
        "workload": f"{len(all_streams)} streams, dim 2/3, W log-uniform 1k..200k (sum "
                    f"{sum(st.window for st in all_streams):,}), S 1-10% of W (sum "
                    f"{sum(st.stride for st in all_streams):,} per round), mixture data, Eps fitted per stream to a mean neighbour count drawn from 10-30",
        "value": value, "unit": UNIT, "rounds": len(timed),
        "round_ms_p50": float(np.percentile(per_round, 50)), "round_ms_p99": float(np.percentile(per_round, 99)),
        "speedup_vs_plain": value / plain_value,
        "plain_one_at_a_time": {"value": plain_value, "round_ms": plain_ms,
                                "config": "autotuned per stream bucket on single-engine slides"},
        "plain_one_at_a_time_default": {"value": default_value, "round_ms": default_ms,
                                        "config": "1 cell per Eps, 8 items per grab, 16 lanes per count query"},
        "launches_per_round": stats["launches_per_round"], "graph_replays": stats["graph_replays"],
        "streams_exact_vs_fp64_oracle": f"{len(all_streams) - int(round(n_diff))}/{len(all_streams)}",
        "mean_neighbours_measured": {"min": round(float(mean_nn.min()), 1),
                                     "median": round(float(np.median(mean_nn)), 1),
                                     "max": round(float(mean_nn.max()), 1),
                                     "streams_in_10_30": f"{int(((mean_nn >= 10) & (mean_nn <= 30)).sum())}/{len(mean_nn)}",
                                     "source": "exact counts of each stream's first window (rank 0's streams)"},
        "streams_per_rank": n_streams, "sharding": f"{world} rank(s), streams partitioned by W, no collective",
        "phase_ms": prof,
        "autotune": {"buckets": len(tuner.cache), "tuned_now": tuner.tuned, "tune_s": round(tuner.tune_seconds, 2),
                     "choices_file": os.path.relpath(choices_file, ROOT)},
    }


def run_serving(args, dev, stream, world=1, rank=0, n_streams=1000, loads=(0.3, 0.6, 0.9), duration=1.5,
                k_slides=4):
    """Continuous-batching server over 1,000 streams (the batched mix),
    Poisson slide requests at offered loads relative to the measured
    all-stream round rate, HBM budget 120 GB; p50/p99 request latency
    (arrival -> completion of its round) and slid points/s.  Then the same
    mix under a budget that holds most streams back (each stream takes three
    requests and leaves, freeing memory for the waiting ones).  With N ranks
    each serves its share of the streams."""
    import torch

    from rtdbstream_gb300 import make_params, stream_bytes
    from rtdbstream_gb300.serve import ServedStream, SlideServer, poisson_arrivals

    all_specs = wl.mixed_streams(n_streams, seed=7)
    # Eps fitted per stream on a 1,000-point sample (the serving leg reports latency,
    # not neighbour counts; the finer fit of the batched leg would add a minute here)
    specs = [wl.calibrate_eps(all_specs[i], n_query=1000)
             for i in partition_streams([s.window for s in all_specs], world, rank)]
    n_mine = len(specs)

    def served(sp):
        pts = wl.mix_points(sp, sp.window + k_slides * sp.stride)
        data = torch.from_numpy(np.ascontiguousarray(pts[sp.window:]).reshape(k_slides, sp.stride * sp.dim)).to(dev)
        return ServedStream(sp, pts[:sp.window], data)

    def combined(r):
        v, _, _ = combine_ranks(r["slid_points_per_s"] * r["wall_s"], 1000.0 * r["wall_s"], world, f"cuda:{dev}")
        _, _, p99 = combine_ranks(0.0, r["latency_ms_p99"], world, f"cuda:{dev}")
        return v, p99

    srv = SlideServer(device=dev, hbm_budget_bytes=120 * 10**9, stream=stream.cuda_stream)
    for sp in specs:
        srv.add(served(sp))
    # capacity: every stream in every round
    t_all = np.zeros(3 * n_mine)
    tgt_all = np.tile(np.arange(n_mine), 3)
    cap = srv.run(t_all, tgt_all)
    cap_rps = cap["requests"] / cap["wall_s"]
    cap_value, _ = combined(cap)
    sweeps = {}
    for depth in (1, 2):  # rounds formed as the previous completes / one queued behind it
        srv.depth = depth
        sweep = []
        for f in loads:
            rate = f * cap_rps
            t, tgt = poisson_arrivals(rate, duration, n_mine, seed=int(f * 100) + 1000 * rank)
            r = srv.run(t, tgt)
            v, p99max = combined(r)
            sweep.append({"offered_requests_per_s": rate * world, "offered_fraction": f, "requests": r["requests"],
                          "slid_points_per_s": v, "latency_ms_p50": r["latency_ms_p50"],
                          "latency_ms_p99": r["latency_ms_p99"], "latency_ms_p99_max_over_ranks": p99max,
                          "mean_round_size": r["mean_round_size"]})
        sweeps[depth] = sweep
    st = srv.pool.stats()
    srv.close()

    # budget-bound: 40% of the mix's memory; each stream takes 3 requests
    costs = [stream_bytes(make_params(sp.dim, sp.window, sp.stride, sp.eps, sp.min_pts)) for sp in specs]
    budget = int(0.4 * sum(costs))
    srv = SlideServer(device=dev, hbm_budget_bytes=budget, stream=stream.cuda_stream)
    streams = [served(sp) for sp in specs]
    for s in streams:
        s.requests_total = 3
        srv.add(s)
    waiting0 = len(srv.waiting)
    t, tgt = poisson_arrivals(0.6 * cap_rps, 3 * n_mine / (0.6 * cap_rps), n_mine, seed=77 + rank)
    # exactly 3 requests per stream: its first 3 Poisson ones, topped up after them
    keep = np.sort(np.concatenate([np.flatnonzero(tgt == i)[:3] for i in range(n_mine)]))
    per = np.bincount(tgt[keep], minlength=n_mine)
    extra = np.repeat(np.arange(n_mine), 3 - per)
    t0 = t[keep].max() if len(keep) else 0.0
    t = np.concatenate([t[keep], t0 + 1e-4 * np.arange(1, len(extra) + 1)])
    tgt = np.concatenate([tgt[keep], extra.astype(tgt.dtype)])
    rb = srv.run(t, tgt)
    vb, p99b = combined(rb)
    done_all = all(s.done == 3 for s in streams)
    srv.close()
    return {"workload": f"{n_streams} streams (the batched mix, W 1k..200k), Poisson slide requests, "
                        f"HBM budget 120 GB ({st['bytes_in_use'] / 1e9:.1f} GB admitted on rank 0); sweep: a round is formed "
                        f"when the previous completes; sweep_pipelined: one more round queued while one runs",
            "capacity_requests_per_s": cap_rps * world, "capacity_slid_points_per_s": cap_value,
            "sweep": sweeps[1],
            "sweep_pipelined": sweeps[2],
            "budget_bound": {"budget_bytes": budget, "mix_bytes": int(sum(costs)),
                             "streams_waiting_at_start": waiting0, "requests": rb["requests"],
                             "all_streams_served_and_retired": done_all,
                             "slid_points_per_s": vb, "latency_ms_p50": rb["latency_ms_p50"],
                             "latency_ms_p99": rb["latency_ms_p99"], "latency_ms_p99_max_over_ranks": p99b,
                             "admission_wait_ms_p50": rb["admission_wait_ms_p50"]}}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
