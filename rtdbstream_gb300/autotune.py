"""Autotuner for a stream's launch configuration.

Three knobs change how the engine works without changing its results:
- ``cell_mult`` (K): grid cells per Eps along each axis.  K = 2 scans the
  (2K+1)^d = 5^d cells of side Eps/2 around a point, which tests fewer pairs
  where cells are dense, but costs more cells, table lookups and work items
  where they are sparse.
- ``work_grab``: work items (cell runs) a clustering warp takes from the
  shared queue at a time -- the work split between warps.  Small grabs balance
  uneven items; large ones keep consecutive cells on one warp and cost fewer
  queue atomics.
- ``query_lanes``: the block shape of the count passes -- 16 lanes per expired
  or new point (two points per warp, 16 per 256-thread block, their dependent
  loads overlapping) or 32 (one point per warp, half the loop trips where
  neighbourhoods are large).  Two cells per Eps always take 32.

Streams are grouped into buckets by dimension, predicate, window size and
density (mean points per occupied Eps-cell of a sample window).  For a
bucket seen for the first time the tuner times every candidate on the
stream's own points and stores the choice in a JSON cache, so later streams
of the bucket, and later runs, reuse it.  A stream slid alone is latency-bound
and one slid in a pool round is throughput-bound, so the two are tuned
apart: `choose` times a single engine (its first window, then a few slides),
`choose_batched` times pool rounds over up to 16 streams of each bucket
together.  The default (one cell per Eps, 8 items per grab) is kept unless a
candidate is at least 3% faster, so timing noise does not pick a
configuration.  Candidates are (cell_mult, work_grab, query_lanes) triples.
"""
from __future__ import annotations

import json
import math
import os
import time
from typing import Callable, Dict, Iterable, Optional, Tuple

import numpy as np

from .engine import Engine, make_params

# (cell_mult, work_grab, query_lanes); the first is the default
CANDIDATES: Tuple[Tuple[int, int, int], ...] = ((1, 8, 16), (1, 5, 16), (1, 4, 16), (1, 16, 16), (1, 2, 16), (1, 1, 16),
                                                (1, 8, 32), (2, 8, 32), (2, 4, 32), (2, 16, 32), (2, 1, 32))
MARGIN = 0.97           # a candidate replaces the default only when this much faster
POOL_STREAMS = 16       # streams of a bucket timed together by choose_batched

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def density(points: np.ndarray, eps: float, sample: int = 200_000) -> float:
    """Mean number of points per occupied cell of side Eps (a sample of at
    most `sample` points, so large windows cost little)."""
    pts = np.asarray(points, dtype=np.float64)
    if len(pts) > sample:
        pts = pts[:sample]
    cells = np.floor((pts - pts.min(axis=0)) / eps).astype(np.int64)
    _, counts = np.unique(cells, axis=0, return_counts=True)
    return float(len(pts) / max(1, len(counts)))


def bucket_key(dim: int, window: int, precision: str, dens: float) -> str:
    """Buckets: powers of two of the window and of the density."""
    wb = int(round(math.log2(max(window, 1))))
    db = int(round(math.log2(max(dens, 1e-3))))
    return f"d{dim}-{precision}-W2^{wb}-n2^{db}"


class Autotuner:
    """Picks (cell_mult, work_grab, query_lanes) per stream bucket.

    `timer(points, dim, W, S, eps, min_pts, precision, cell_mult, work_grab,
    query_lanes)` returns milliseconds per slide; the default times real slides
    on the GPU.  `pool_timer(streams, cell_mult, work_grab, query_lanes)` does
    the same for pool rounds.
    """

    def __init__(self, cache_path: Optional[str] = None, device: int = 0, slides: int = 4,
                 candidates: Iterable[Tuple[int, int]] = CANDIDATES, timer: Optional[Callable] = None,
                 pool_timer: Optional[Callable] = None):
        self.cache_path = cache_path or os.environ.get("RTDBS_AUTOTUNE_CACHE") or DEFAULT_CACHE
        self.device = device
        self.slides = slides
        self.candidates = tuple(candidates)
        self.timer = timer or self._time_on_gpu
        self.pool_timer = pool_timer or self._time_pool_on_gpu
        self.cache: Dict[str, dict] = {}
        self.tuned = 0           # buckets timed in this process
        self.tune_seconds = 0.0
        if os.path.exists(self.cache_path):
            try:
                with open(self.cache_path) as f:
                    self.cache = json.load(f)
            except (OSError, ValueError):
                self.cache = {}

    def choose(self, points: np.ndarray, dim: int, window: int, stride: int, eps: float, min_pts: int,
               precision: str = "fp64") -> dict:
        """The bucket's configuration: {"cell_mult", "work_grab", "query_lanes", "ms"}."""
        key = bucket_key(dim, window, precision, density(points[:window], eps))
        hit = self.cache.get(key)
        if hit is not None and "query_lanes" in hit:
            return hit
        return self._tune(key, lambda km, grab, ql: self.timer(points, dim, window, stride, eps, min_pts,
                                                                 precision, km, grab, ql))

    def choose_batched(self, streams) -> list:
        """Configurations for streams slid together in pool rounds.  `streams`
        holds (points, dim, window, stride, eps, min_pts, precision) tuples
        (points: a window and a few strides); returns one configuration per
        stream, tuned per bucket on pool rounds of the bucket's streams."""
        keys = [("pool:" + bucket_key(st[1], st[2], st[6], density(st[0][:st[2]], st[4]))) for st in streams]
        groups: Dict[str, list] = {}
        for k, st in zip(keys, streams):
            groups.setdefault(k, []).append(st)
        for k, members in groups.items():
            if "query_lanes" not in self.cache.get(k, {}):
                sel = members[:POOL_STREAMS]
                self._tune(k, lambda km, grab, ql: self.pool_timer(sel, km, grab, ql))
        return [self.cache[k] for k in keys]

    def _tune(self, key: str, run: Callable) -> dict:
        t0 = time.perf_counter()
        ms = {}
        for km, grab, ql in self.candidates:
            try:
                ms[f"{km},{grab},{ql}"] = float(run(km, grab, ql))
            except Exception:  # a configuration the stream cannot take is skipped
                continue
        if not ms:
            raise RuntimeError(f"autotune: no candidate configuration ran for bucket {key}")
        best = min(ms, key=ms.get)
        default = "{},{},{}".format(*self.candidates[0])
        if default in ms and ms[best] > MARGIN * ms[default]:
            best = default
        km, grab, ql = (int(x) for x in best.split(","))
        self.cache[key] = {"cell_mult": km, "work_grab": grab, "query_lanes": ql, "ms": ms}
        self.tuned += 1
        self.tune_seconds += time.perf_counter() - t0
        self._save()
        return self.cache[key]

    def params(self, points: np.ndarray, dim: int, window: int, stride: int, eps: float, min_pts: int,
               precision: str = "fp64", **kw):
        """rtdbs_params of a stream with the tuned configuration."""
        c = self.choose(points, dim, window, stride, eps, min_pts, precision)
        return make_params(dim, window, stride, eps, min_pts, precision=precision, cell_mult=c["cell_mult"],
                           work_grab=c["work_grab"], query_lanes=c["query_lanes"], **kw)

    def _save(self) -> None:
        d = os.path.dirname(self.cache_path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.cache, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def _time_on_gpu(self, points, dim, window, stride, eps, min_pts, precision, cell_mult, work_grab,
                     query_lanes):
        import torch

        need = window + (self.slides + 1) * stride
        if len(points) < need:
            raise ValueError("autotune: the sample needs a window and a few strides of points")
        dev = torch.device("cuda", self.device)
        s = torch.cuda.Stream(device=dev)
        d = torch.from_numpy(np.ascontiguousarray(points[window:need], dtype=np.float32)).to(dev)
        torch.cuda.synchronize(dev)  # the copy is on torch's stream, the slides on s
        with torch.cuda.stream(s):
            with Engine(dim, window, stride, eps, min_pts, precision=precision, device=self.device,
                        stream=s.cuda_stream, cell_mult=cell_mult, work_grab=work_grab,
                        query_lanes=query_lanes) as eng:
                eng.load_window(points[:window])
                eng.slide_async(d[:stride])   # warm-up (and the graph capture)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                for k in range(1, self.slides + 1):
                    eng.slide_async(d[k * stride:(k + 1) * stride])
                b.record(s)
                eng.sync()
                return a.elapsed_time(b) / self.slides

    def _time_pool_on_gpu(self, streams, cell_mult, work_grab, query_lanes, rounds: int = 3):
        import torch

        from .engine import Pool

        dev = torch.device("cuda", self.device)
        s = torch.cuda.Stream(device=dev)
        need = rounds + 2
        for pts, dim, W, S, eps, mp, prec in streams:
            if len(pts) < W + need * S:
                raise ValueError("autotune: the sample needs a window and a few strides of points")
        packed = [torch.from_numpy(np.concatenate([np.ascontiguousarray(pts[W + k * S: W + (k + 1) * S],
                                                                        dtype=np.float32).reshape(-1)
                                                   for pts, dim, W, S, eps, mp, prec in streams])).to(dev)
                  for k in range(need)]
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(s):
            with Pool(device=self.device, use_graph=True, stream=s.cuda_stream) as pool:
                ids = []
                for pts, dim, W, S, eps, mp, prec in streams:
                    sid = pool.add_stream(make_params(dim, W, S, eps, mp, precision=prec, device=self.device,
                                                      cell_mult=cell_mult, work_grab=work_grab,
                                                      query_lanes=query_lanes))
                    pool.load_window(sid, pts[:W])
                    ids.append(sid)
                pool.slide(ids, packed[0])
                pool.slide(ids, packed[1])   # warm-up and the graph capture
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                for k in range(2, need):
                    pool.slide(ids, packed[k])
                b.record(s)
                pool.sync()
                return a.elapsed_time(b) / rounds
