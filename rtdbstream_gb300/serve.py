"""Continuous-batching slide server on a stream pool.

Many streams share one GPU.  Clients send slide requests (a stream id and its
next S points); the server keeps every admitted stream's window, grid, counts
and forest resident in HBM and runs rounds back to back.  Each round takes the
oldest pending request of every stream that has one, so requests that arrive
while a round is on the GPU join a following round instead of waiting for a
fixed batch.  With depth > 1 rounds are pipelined: while one round runs on
the GPU the host builds and queues the next (up to `depth` rounds in flight
on the pool's CUDA stream, which keeps each stream's slides in order), so
building a round does not leave the GPU idle; each queued round also has a
fixed cost, so at light load depth 1 (a round is formed when the previous
one completes) gives the lower latency.  Streams are admitted against an HBM budget and
wait for memory when it is exhausted; a stream that has had all its slides
leaves and frees its memory.  Latency of a request = completion of its round
(its CUDA event) - its arrival.
"""
from __future__ import annotations

import collections
import gc
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .engine import Pool, RtdbsError, RTDBS_ERR_BUDGET, make_params, stream_bytes


@dataclass
class ServedStream:
    spec: object                   # dim, window, stride, eps, min_pts
    window_points: np.ndarray      # first window, host [W, dim]
    slide_data: object             # device tensor [k_slides, S * dim]
    requests_total: int = 0        # slides this stream will receive (0: no limit)
    sid: Optional[int] = None      # pool slot while admitted
    done: int = 0                  # slides completed
    issued: int = 0                # slides queued on the GPU (selects the input row)
    pending: collections.deque = field(default_factory=collections.deque)


class SlideServer:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 120 * 10**9, stream: int = 0, depth: int = 1):
        self.pool = Pool(device=device, hbm_budget_bytes=hbm_budget_bytes, use_graph=False, stream=stream)
        self.budget = hbm_budget_bytes
        self.depth = max(1, depth)
        self.streams: List[ServedStream] = []
        self.waiting = collections.deque()   # streams not yet admitted (budget)
        self.rounds = 0
        self.round_sizes = []
        self.admit_waits = []                # seconds between a stream's first request and its admission

    def close(self):
        self.pool.close()

    def add(self, s: ServedStream) -> None:
        """Queues a stream for admission; one that alone exceeds the whole
        HBM budget is refused at once (RTDBS_ERR_BUDGET)."""
        sp = s.spec
        need = stream_bytes(make_params(sp.dim, sp.window, sp.stride, sp.eps, sp.min_pts))
        if self.budget and need > self.budget:
            raise RtdbsError(RTDBS_ERR_BUDGET, f"stream needs {need} bytes, more than the whole budget "
                                               f"of {self.budget}")
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
        self.round_sizes = []
        self.admit_waits = []
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

        cuda_stream = torch.cuda.current_stream()
        t0 = time.perf_counter()
        inflight = collections.deque()    # (event, members, arrival times) per queued round
        first_req = {}                    # waiting stream -> time of its first request
        while True:
            now = time.perf_counter() - t0
            while nxt < n and arrivals[nxt] <= now:
                i = int(targets[nxt])
                self.streams[i].pending.append(arrivals[nxt])
                active.add(i)
                if self.streams[i].sid is None:
                    first_req.setdefault(i, arrivals[nxt])
                nxt += 1
            # rounds the GPU has finished, oldest first: their requests complete
            while inflight and inflight[0][0].query():
                _, members, arr = inflight.popleft()
                done_t = time.perf_counter() - t0
                for i, a in zip(members, arr):
                    s = self.streams[i]
                    s.done += 1
                    slid += s.spec.stride
                    lat.append(done_t - a)
                    if s.requests_total and s.done >= s.requests_total:
                        was_waiting = set(self.waiting)
                        self._retire(i)
                        active.discard(i)
                        s.pending.clear()                          # beyond its total: never served
                        for j in was_waiting - set(self.waiting):  # admitted by the freed memory
                            if j in first_req:
                                self.admit_waits.append(done_t - first_req.pop(j))
            if len(inflight) < self.depth:
                members = [i for i in active if self.streams[i].sid is not None]
                if members:
                    ids, ptrs, arr = [], [], []
                    for i in members:
                        s = self.streams[i]
                        ids.append(s.sid)
                        ptrs.append(base[i] + (s.issued % krow[i]) * row[i])
                        s.issued += 1
                        arr.append(s.pending.popleft())
                        if not s.pending:
                            active.discard(i)
                    self.pool.slide_each(ids, ptrs)
                    ev = torch.cuda.Event()
                    ev.record(cuda_stream)
                    inflight.append((ev, members, arr))
                    self.rounds += 1
                    self.round_sizes.append(len(members))
                    continue
            if not inflight:  # (and no admitted stream has a pending request)
                if nxt >= n and not active:
                    break
                if nxt >= n:
                    # only streams that wait for admission have requests, and
                    # no round, arrival or departure can free memory for them
                    raise RtdbsError(RTDBS_ERR_BUDGET, f"{len(active)} stream(s) with pending requests wait "
                                                       "for admission and nothing in flight can free memory")
                delay = arrivals[nxt] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(min(delay, 1e-3))
        wall = time.perf_counter() - t0
        self.pool.sync()
        return {"requests": len(lat), "wall_s": wall, "slid_points_per_s": slid / wall,
                "latency_ms_p50": 1000 * float(np.percentile(lat, 50)) if lat else None,
                "latency_ms_p99": 1000 * float(np.percentile(lat, 99)) if lat else None,
                "rounds": self.rounds, "mean_round_size": float(np.mean(self.round_sizes)) if lat else 0.0,
                "admission_wait_ms_p50": 1000 * float(np.percentile(self.admit_waits, 50))
                if self.admit_waits else None}


def poisson_arrivals(rate: float, duration: float, n_streams: int, seed: int = 0):
    """Request times (Poisson process of `rate` per second over `duration`)
    and uniformly chosen target streams."""
    rng = np.random.default_rng(seed)
    n = rng.poisson(rate * duration)
    t = np.sort(rng.uniform(0.0, duration, n))
    return t, rng.integers(0, n_streams, n)
