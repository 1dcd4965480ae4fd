"""Continuous-batching slide server on a stream pool.

Many streams share one GPU.  Clients send slide requests (a stream id and its
next S points); the server keeps every admitted stream's window, grid, counts
and forest resident in HBM and runs rounds back to back.  Each round takes the
oldest pending request of every stream that has one, so requests that arrive
while a round is on the GPU join the next round instead of waiting for a
fixed batch.  Streams are admitted against an HBM budget and wait for memory
when it is exhausted; a stream that has had all its slides leaves and frees
its memory.  Latency of a request = completion of its round - its arrival.
"""
from __future__ import annotations

import collections
import gc
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .engine import Pool, RtdbsError, RTDBS_ERR_BUDGET, make_params


@dataclass
class ServedStream:
    spec: object                   # dim, window, stride, eps, min_pts
    window_points: np.ndarray      # first window, host [W, dim]
    slide_data: object             # device tensor [k_slides, S * dim]
    requests_total: int = 0        # slides this stream will receive
    sid: Optional[int] = None      # pool slot while admitted
    done: int = 0
    pending: collections.deque = field(default_factory=collections.deque)


class SlideServer:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 120 * 10**9, stream: int = 0):
        self.pool = Pool(device=device, hbm_budget_bytes=hbm_budget_bytes, use_graph=False, stream=stream)
        self.streams: List[ServedStream] = []
        self.waiting = collections.deque()   # streams not yet admitted (budget)
        self.rounds = 0
        self.round_sizes = []

    def close(self):
        self.pool.close()

    def add(self, s: ServedStream) -> None:
        self.streams.append(s)
        self.waiting.append(len(self.streams) - 1)
        self._admit()

    def _admit(self) -> None:
        while self.waiting:
            i = self.waiting[0]
            s = self.streams[i]
            sp = s.spec
            try:
                s.sid = self.pool.add_stream(make_params(sp.dim, sp.window, sp.stride, sp.eps, sp.min_pts))
            except RtdbsError as e:
                if e.status == RTDBS_ERR_BUDGET:
                    return            # admitted when memory frees up
                raise
            self.pool.load_window(s.sid, s.window_points)
            self.waiting.popleft()

    def _retire(self, i: int) -> None:
        s = self.streams[i]
        self.pool.remove_stream(s.sid)
        s.sid = None
        self._admit()

    def run(self, arrivals: np.ndarray, targets: np.ndarray) -> dict:
        """Serve requests arriving at `arrivals` (seconds from the start,
        sorted) for stream indices `targets`; returns latency and throughput.
        The pool's CUDA stream must be torch's current stream."""
        base = [s.slide_data.data_ptr() for s in self.streams]
        row = [s.slide_data.shape[1] * s.slide_data.element_size() for s in self.streams]
        krow = [s.slide_data.shape[0] for s in self.streams]
        lat = []
        slid = 0
        n = len(arrivals)
        nxt = 0
        active = set()                  # streams with pending requests
        # no collector pauses inside the request loop (they would show as
        # latency spikes); collect once the run is over
        gc_was_on = gc.isenabled()
        gc.disable()
        try:
            return self._loop(arrivals, targets, base, row, krow, lat, slid, n, nxt, active)
        finally:
            if gc_was_on:
                gc.enable()

    def _loop(self, arrivals, targets, base, row, krow, lat, slid, n, nxt, active) -> dict:
        import torch

        t0 = time.perf_counter()
        while True:
            now = time.perf_counter() - t0
            while nxt < n and arrivals[nxt] <= now:
                i = int(targets[nxt])
                self.streams[i].pending.append(arrivals[nxt])
                active.add(i)
                nxt += 1
            members = [i for i in active if self.streams[i].sid is not None]
            if not members:
                if nxt >= n and not active:
                    break
                if nxt < n:
                    delay = arrivals[nxt] - (time.perf_counter() - t0)
                    if delay > 0:
                        time.sleep(min(delay, 1e-3))
                continue
            ids, ptrs, arr = [], [], []
            for i in members:
                s = self.streams[i]
                ids.append(s.sid)
                ptrs.append(base[i] + (s.done % krow[i]) * row[i])
                arr.append(s.pending.popleft())
                if not s.pending:
                    active.discard(i)
            self.pool.slide_each(ids, ptrs)
            ev = torch.cuda.Event()
            ev.record(torch.cuda.current_stream())
            while not ev.query():
                pass
            done_t = time.perf_counter() - t0
            self.rounds += 1
            self.round_sizes.append(len(members))
            for i, a in zip(members, arr):
                s = self.streams[i]
                s.done += 1
                slid += s.spec.stride
                lat.append(done_t - a)
                if s.requests_total and s.done >= s.requests_total:
                    self._retire(i)
                    active.discard(i)
        wall = time.perf_counter() - t0
        self.pool.sync()
        return {"requests": len(lat), "wall_s": wall, "slid_points_per_s": slid / wall,
                "latency_ms_p50": 1000 * float(np.percentile(lat, 50)) if lat else None,
                "latency_ms_p99": 1000 * float(np.percentile(lat, 99)) if lat else None,
                "rounds": self.rounds, "mean_round_size": float(np.mean(self.round_sizes)) if lat else 0.0}


def poisson_arrivals(rate: float, duration: float, n_streams: int, seed: int = 0):
    """Request times (Poisson process of `rate` per second over `duration`)
    and uniformly chosen target streams."""
    rng = np.random.default_rng(seed)
    n = rng.poisson(rate * duration)
    t = np.sort(rng.uniform(0.0, duration, n))
    return t, rng.integers(0, n_streams, n)
