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
e2e    -- rtdbs_slide with pinned host buffers: H2D of S points, the slide,
          D2H of label[W] and cluster_id[W], host wall clock per call.
With N > 1 (torchrun), every rank slides its own stream (seed + rank): the
path shards by stream with no collective (weak scaling).

--impl reference: the reference's CPU path (cluster_with_cpu,
src/dbscan/util.cpp:299-354, through the oracle's restatement) on the host
cores, projected from bounded sub-window samples (it is O(W^2) per slide).
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


def walker_stream(n_total: int, seed: int) -> np.ndarray:
    """The walker stream; a smaller window keeps 500 points per walker trail
    (2,000 walkers at W = 1M), so the local density matches the full size."""
    walkers = max(1, round(2000 * SPEC.window / 1_000_000))
    return wl.random_walkers(n_total, n_walkers=walkers, seed=seed)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ------------------------------------------------------------ CPU reference

def cpu_reference_sample(points: np.ndarray, threads: int, budget_s: float = 12.0) -> dict:
    """The reference's CPU path (restated cluster_with_cpu, FP32, O(W^2)) on
    sub-windows of the benchmark stream; slid points/s projected to the full
    window by the W^2 cost law (its pair loop is exactly W(W-1)/2 tests)."""
    import concurrent.futures as cf

    import oracle

    oracle.build(ref=False)
    W, S = SPEC.window, SPEC.stride
    sub = 16384
    # calibrate: one sample, then as many rounds as the budget allows
    def one(k):
        win = oracle.window_of(points, W, S, k)[:sub]
        t0 = time.perf_counter()
        oracle.window_bruteforce(win, SPEC.eps, SPEC.min_pts)
        return time.perf_counter() - t0

    avail = (len(points) - W) // S
    if avail < 1:
        raise ValueError("stream too short for one slide")
    t1 = one(1)
    rounds = max(1, int(budget_s / max(t1, 1e-3)))
    jobs = [1 + (i % avail) for i in range(rounds * threads)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        per = list(ex.map(one, jobs))
    wall = time.perf_counter() - t0
    mean_sample = statistics.mean(per)
    scale = (W / sub) ** 2
    # slides completed per second by `threads` cores at full W
    value = threads * S / (mean_sample * scale)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"restated cluster_with_cpu on {len(per)} sub-windows of {sub} points of the "
                       f"walker stream ({wall:.1f} s wall on {threads} thread(s), mean {mean_sample:.3f} "
                       f"s/sample), projected to W={W} by (W/{sub})^2")}


def run_reference(args) -> None:
    world, rank, _ = dist_env()
    if rank != 0:
        return
    pts = walker_stream(SPEC.window + 60 * SPEC.stride, seed=1)
    threads = os.cpu_count() or 1
    base = cpu_reference_sample(pts, threads)
    steps = max(1, args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * SPEC.stride / base["value"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "window": SPEC.window, "stride": SPEC.stride,
                   "eps": SPEC.eps, "min_pts": SPEC.min_pts, "dim": 3},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- our engine

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
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
        "merge": W * (28 + 28 + 4) + c * (8 + 16),
        "build": W * 8 + cells * 32 + items * 8,
        "increment": c * (8 + 16) + c * 4,
        "union": W * (16 + 4 + 4 + 4),
        # scnt, slot, root hint, parent read; root by slot written
        "flatten": W * (4 + 4 + 4 + 4 + 4),
        # border pass: root by slot read; label, cid, parent written
        "label": W * (4 + 4 + 4 + 4),
    }[phase]


def measured_peak() -> tuple:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(phase: str):
    """DRAM bytes per launch of the dominant kernel at W = 1M from the
    committed ncu summary (profiles/ncu_traffic.json, a W = 250k capture
    scaled by 4), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get({"label": "k_border"}.get(phase, f"k_{phase}"))
    except (OSError, ValueError):
        return None


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
    total_steps = args.warmup + args.steps + args.e2e_steps + args.profile_steps
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
    with ClockSampler(dev) as clk:
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
    e2e_value = S / statistics.mean(e2e_s) if e2e_s else None

    # per-phase device times (direct launches bracketed by events)
    prof = []
    for _ in range(args.profile_steps):
        flush.fill_(2.0)
        prof.append(eng.slide_profiled(new_pts(step)))
        step += 1
    st = eng.stats()
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

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    peak, peak_kind = measured_peak()
    dom = max(avg, key=avg.get) if avg else None
    roofline = None
    if dom:
        launches = st["chunks_per_slide"] if dom not in ("union", "flatten", "label") else 1
        alg = algorithmic_bytes(dom, W, S, 3, st["cells"], st["work_items"]) * launches
        achieved = alg / (avg[dom] / 1000.0) / 1e9
        slide_alg = sum(algorithmic_bytes(p, W, S, 3, st["cells"], st["work_items"]) for p in phases)
        roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                    "traffic": ncu_traffic(dom), "algorithmic_bytes_per_launch": alg,
                    "phase_ms": avg,
                    "slide": {"algorithmic_bytes": slide_alg,
                              "achieved_gbs": slide_alg / (total_ms / args.steps / 1000.0) / 1e9,
                              "frac": slide_alg / (total_ms / args.steps / 1000.0) / 1e9 / peak}}
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_reference_sample(pts, 1, budget_s=10.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "window": W, "stride": S, "eps": SPEC.eps,
                   "min_pts": SPEC.min_pts, "dim": 3, "precision": "fp64 (fp32 filter + fp64 band)",
                   "l2": "flushed between steps (256 MB write outside the timed events)",
                   "parallelism": f"{world} independent stream(s), one per GPU"},
        "latency_ms": {"p50": float(np.percentile(per_ms, 50)), "p99": float(np.percentile(per_ms, 99))},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": S * 3 * 4,
                "d2h_bytes_per_step": 2 * W * 4,
                "latency_ms_p50": 1000 * float(np.percentile(e2e_s, 50)) if e2e_s else None},
        "gpu_launches": args.steps * st["launches_per_slide"],
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "exact_vs_fp64_oracle": verified,
        "band_rechecks": st["band_rechecks"],
        "dist_tests_per_slide": st["dist_tests"] / max(1, st["slides"]),
    }
    if not args.no_batched and world == 1:
        del d_pts
        line["batched"] = run_batched(args, dev, stream, flush)
    if not args.no_serving and world == 1:
        line["serving"] = run_serving(args, dev, stream)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batched(args, dev, stream, flush, n_streams=256, rounds=None, plain_rounds=4):
    """256 uneven streams slid together by a pool (one launch per phase, a
    CUDA-graph replay per round) against the same streams slid one at a time
    by single-stream engines.  Device-resident inputs, CUDA events per round,
    L2 flushed between rounds outside the events."""
    import torch

    from rtdbstream_gb300 import Engine, Pool, make_params

    streams = wl.mixed_streams(n_streams)
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
    value = slid * len(timed) / (sum(per_round) / 1000.0)
    # exactness of a sample of streams against the FP64 oracle
    import oracle

    oracle.build(ref=False)
    exact = True
    for i in range(0, n_streams, max(1, n_streams // 8)):
        st = streams[i]
        win = oracle.window_of(data[i], st.window, st.stride, rounds)
        _, elab, ecid, _ = oracle.window_grid(win, st.eps, st.min_pts, oracle.MODE_FP64)
        lab, cid = pool.outputs(ids[i])
        exact = exact and bool(np.array_equal(lab, elab) and np.array_equal(cid, ecid))
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

    plain_ms = [plain_round_ms(tuned_plain)]
    default_ms = plain_round_ms([{"cell_mult": 1, "work_grab": 8, "query_lanes": 16}] * len(streams))
    plain_value = slid / (statistics.mean(plain_ms) / 1000.0)
    return {
        "workload": f"{n_streams} streams, dim 2/3, W log-uniform 1k..200k (sum {sum(st.window for st in streams):,}),"
                    f" S 1-10% of W (sum {slid:,} per round), mixture data, Eps for 10-30 mean neighbours",
        "value": value, "unit": UNIT, "rounds": len(timed),
        "round_ms_p50": float(np.percentile(per_round, 50)), "round_ms_p99": float(np.percentile(per_round, 99)),
        "plain_one_at_a_time": {"value": plain_value, "round_ms": statistics.mean(plain_ms),
                                "config": "autotuned per stream bucket on single-engine slides"},
        "plain_one_at_a_time_default": {"value": slid / (default_ms / 1000.0), "round_ms": default_ms,
                                        "config": "1 cell per Eps, 8 items per grab, 16 lanes per count query"},
        "speedup_vs_plain": value / plain_value,
        "launches_per_round": stats["launches_per_round"], "graph_replays": stats["graph_replays"],
        "phase_ms": prof,
        "exact_sample_vs_fp64_oracle": exact,
        "autotune": {"buckets": len(tuner.cache), "tuned_now": tuner.tuned, "tune_s": round(tuner.tune_seconds, 2),
                     "choices": {k: [v["cell_mult"], v["work_grab"], v.get("query_lanes")]
                                 for k, v in sorted(tuner.cache.items())
                                 if k.startswith("pool:")},
                     "plain_choices": {k: [v["cell_mult"], v["work_grab"], v.get("query_lanes")]
                                       for k, v in sorted(tuner.cache.items())
                                       if not k.startswith("pool:")}},
    }


def run_serving(args, dev, stream, n_streams=1000, loads=(0.3, 0.6, 0.9), duration=1.5, k_slides=4):
    """Continuous-batching server over 1,000 streams (the batched mix),
    Poisson slide requests at offered loads relative to the measured
    all-stream round rate, HBM budget 120 GB; p50/p99 request latency
    (arrival -> completion of its round) and slid points/s."""
    import torch

    from rtdbstream_gb300.serve import ServedStream, SlideServer, poisson_arrivals

    specs = wl.mixed_streams(n_streams, seed=7)
    srv = SlideServer(device=dev, hbm_budget_bytes=120 * 10**9, stream=stream.cuda_stream)
    for sp in specs:
        pts = wl.mix_points(sp, sp.window + k_slides * sp.stride)
        data = torch.from_numpy(np.ascontiguousarray(pts[sp.window:]).reshape(k_slides, sp.stride * sp.dim)).to(dev)
        srv.add(ServedStream(sp, pts[:sp.window], data))
    # capacity: every stream in every round
    t_all = np.zeros(3 * n_streams)
    tgt_all = np.tile(np.arange(n_streams), 3)
    cap = srv.run(t_all, tgt_all)
    cap_rps = cap["requests"] / cap["wall_s"]
    sweep = []
    for f in loads:
        rate = f * cap_rps
        t, tgt = poisson_arrivals(rate, duration, n_streams, seed=int(f * 100))
        r = srv.run(t, tgt)
        sweep.append({"offered_requests_per_s": rate, "offered_fraction": f,
                      **{k: r[k] for k in ("requests", "slid_points_per_s", "latency_ms_p50", "latency_ms_p99",
                                           "mean_round_size")}})
    st = srv.pool.stats()
    srv.close()
    return {"workload": f"{n_streams} streams (the batched mix, W 1k..200k), Poisson slide requests, "
                        f"HBM budget 120 GB ({st['bytes_in_use'] / 1e9:.1f} GB admitted)",
            "capacity_requests_per_s": cap_rps, "capacity_slid_points_per_s": cap["slid_points_per_s"],
            "sweep": sweep}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
