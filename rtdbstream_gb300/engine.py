"""ctypes binding of the C ABI (include/rtdbs.h) and a thin Python engine.

The Python names follow the reference's ScanState fields (window_size,
stride_size, radius, min_pts; src/dbscan/state.h:61-67) and its driver
(dbscan(), src/dbscan/dbscan.cpp:2258-2364).  Everything numeric runs in
librtdbs.so; there is no Python or CPU fallback: without the library the
constructor raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Tuple

import numpy as np

from . import build as _build

RTDBS_OK = 0
RTDBS_ERR_INVALID = -1
RTDBS_ERR_CUDA = -2
RTDBS_ERR_OOM = -3
RTDBS_ERR_STATE = -4
RTDBS_ERR_DEVICE = -5
RTDBS_ERR_NO_DEVICE = -6
PREC_FP64 = 0
PREC_FP32 = 1
FLAG_NO_GRAPH = 1

EXPORTED_SYMBOLS = (
    "rtdbs_abi_version", "rtdbs_status_string", "rtdbs_last_error", "rtdbs_params_init",
    "rtdbs_create", "rtdbs_destroy", "rtdbs_load_window", "rtdbs_slide", "rtdbs_slide_async",
    "rtdbs_slide_pipelined",
    "rtdbs_sync", "rtdbs_cluster", "rtdbs_get_counts", "rtdbs_device_outputs", "rtdbs_get_stats",
    "rtdbs_slide_profiled", "rtdbs_cluster_window_noalloc", "rtdbs_cluster_window_noalloc_async",
    "rtdbs_stream_bytes", "rtdbs_pool_params_init", "rtdbs_pool_create", "rtdbs_pool_destroy",
    "rtdbs_pool_add_stream", "rtdbs_pool_remove_stream", "rtdbs_pool_load_window", "rtdbs_pool_slide",
    "rtdbs_pool_sync", "rtdbs_pool_outputs", "rtdbs_pool_read_outputs", "rtdbs_pool_engine",
    "rtdbs_pool_get_stats", "rtdbs_pool_slide_profiled", "rtdbs_pool_slide_each", "rtdbs_read_points",
)
RTDBS_ERR_BUDGET = -7


class Params(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("window", ctypes.c_int32), ("stride", ctypes.c_int32),
                ("min_pts", ctypes.c_int32), ("eps", ctypes.c_double), ("precision", ctypes.c_int32),
                ("has_bbox", ctypes.c_int32), ("bbox_min", ctypes.c_float * 3),
                ("bbox_max", ctypes.c_float * 3), ("device", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("cell_mult", ctypes.c_int32), ("work_grab", ctypes.c_int32),
                ("query_lanes", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]


class Stats(ctypes.Structure):
    _fields_ = [("slides", ctypes.c_int64), ("band_rechecks", ctypes.c_int64),
                ("cells", ctypes.c_int64), ("work_items", ctypes.c_int64),
                ("error_bits", ctypes.c_int32), ("key_bits", ctypes.c_int32),
                ("cell_side", ctypes.c_double), ("device_bytes", ctypes.c_int64),
                ("launches_per_slide", ctypes.c_int32), ("chunks_per_slide", ctypes.c_int32),
                ("dist_tests", ctypes.c_int64), ("reused_cores", ctypes.c_int64),
                ("query_tests", ctypes.c_int64), ("query_hits", ctypes.c_int64),
                ("cluster_tests", ctypes.c_int64), ("cluster_hits", ctypes.c_int64),
                ("max_query_tests", ctypes.c_int32), ("reserved0", ctypes.c_int32),
                ("reserved", ctypes.c_int64 * 3)]


PHASES = ("ingest", "sort", "decrement", "merge", "build", "increment", "union", "flatten", "label")


class PhaseTimes(ctypes.Structure):
    _fields_ = [(f"{p}_ms", ctypes.c_float) for p in PHASES] + [
        ("total_ms", ctypes.c_float), ("chunks", ctypes.c_int32)]


class PoolParams(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("flags", ctypes.c_int32), ("max_streams", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("reserved", ctypes.c_int64 * 6)]


class PoolStats(ctypes.Structure):
    _fields_ = [("streams", ctypes.c_int64), ("bytes_in_use", ctypes.c_int64), ("budget_bytes", ctypes.c_int64),
                ("rounds", ctypes.c_int64), ("graph_replays", ctypes.c_int64),
                ("launches_per_round", ctypes.c_int32), ("reserved0", ctypes.c_int32),
                ("reserved", ctypes.c_int64 * 4)]


class RtdbsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"rtdbs status {status}: {msg}")
        self.status = status


_lib = None


def load_library(path: Optional[str] = None) -> ctypes.CDLL:
    """Loads librtdbs.so (building it with nvcc when stale or absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"engine library missing: {path}")
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.rtdbs_abi_version.restype = ctypes.c_int
    L.rtdbs_status_string.restype = ctypes.c_char_p
    L.rtdbs_status_string.argtypes = [ctypes.c_int]
    L.rtdbs_last_error.restype = ctypes.c_char_p
    L.rtdbs_params_init.argtypes = [ctypes.POINTER(Params)]
    L.rtdbs_create.argtypes = [ctypes.POINTER(Params), vp, ctypes.POINTER(vp)]
    L.rtdbs_destroy.argtypes = [vp]
    L.rtdbs_load_window.argtypes = [vp, vp, ctypes.c_int]
    L.rtdbs_slide.argtypes = [vp, vp, vp, vp]
    L.rtdbs_slide_async.argtypes = [vp, vp, vp, vp]
    L.rtdbs_slide_pipelined.argtypes = [vp, vp, vp, vp]
    L.rtdbs_sync.argtypes = [vp]
    L.rtdbs_cluster.argtypes = [vp, vp, vp, ctypes.c_int]
    L.rtdbs_get_counts.argtypes = [vp, vp, ctypes.c_int]
    L.rtdbs_device_outputs.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.rtdbs_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.rtdbs_slide_profiled.argtypes = [vp, vp, ctypes.POINTER(PhaseTimes)]
    L.rtdbs_stream_bytes.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_int64)]
    L.rtdbs_pool_params_init.argtypes = [ctypes.POINTER(PoolParams)]
    L.rtdbs_pool_create.argtypes = [ctypes.POINTER(PoolParams), vp, ctypes.POINTER(vp)]
    L.rtdbs_pool_destroy.argtypes = [vp]
    L.rtdbs_pool_add_stream.argtypes = [vp, ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_int32)]
    L.rtdbs_pool_remove_stream.argtypes = [vp, ctypes.c_int32]
    L.rtdbs_pool_load_window.argtypes = [vp, ctypes.c_int32, vp, ctypes.c_int]
    L.rtdbs_pool_slide.argtypes = [vp, ctypes.c_int32, vp, vp]
    L.rtdbs_pool_sync.argtypes = [vp]
    L.rtdbs_pool_outputs.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.rtdbs_pool_read_outputs.argtypes = [vp, ctypes.c_int32, vp, vp, ctypes.c_int]
    L.rtdbs_pool_engine.argtypes = [vp, ctypes.c_int32, ctypes.POINTER(vp)]
    L.rtdbs_pool_get_stats.argtypes = [vp, ctypes.POINTER(PoolStats)]
    L.rtdbs_pool_slide_profiled.argtypes = [vp, ctypes.c_int32, vp, vp, ctypes.POINTER(PhaseTimes)]
    L.rtdbs_pool_slide_each.argtypes = [vp, ctypes.c_int32, vp, vp]
    L.rtdbs_read_points.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int64, vp,
                                    ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32), vp, vp]
    for name in EXPORTED_SYMBOLS:
        getattr(L, name).restype = getattr(L, name).restype or ctypes.c_int
    _lib = L
    return L


def _check(status: int) -> None:
    if status != RTDBS_OK:
        L = load_library()
        raise RtdbsError(status, L.rtdbs_last_error().decode() or L.rtdbs_status_string(status).decode())


def _ptr(a) -> int:
    """Address of a numpy array or a torch tensor (host or device)."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())


class Engine:
    """One sliding window of `window_size` points, sliding by `stride_size`.

    radius is Eps and min_pts is MinPts (the reference's -R and -K).  Points
    are float32 [n, dim].  Outputs are indexed by ring slot, as in the
    reference: after s slides, stream point t sits in slot t mod window_size.
    """

    def __init__(self, dim: int, window_size: int, stride_size: int, radius: float, min_pts: int,
                 precision: str = "fp64", bbox: Optional[Tuple] = None, device: int = 0,
                 use_graph: bool = True, stream: int = 0, cell_mult: int = 1, work_grab: int = 0,
                 query_lanes: int = 0):
        self._lib = load_library()
        p = make_params(dim, window_size, stride_size, radius, min_pts, precision=precision, bbox=bbox,
                        device=device, use_graph=use_graph, cell_mult=cell_mult, work_grab=work_grab,
                        query_lanes=query_lanes)
        self.params = p
        self.dim, self.window_size, self.stride_size = p.dim, p.window, p.stride
        self.radius, self.min_pts = p.eps, p.min_pts
        h = ctypes.c_void_p()
        _check(self._lib.rtdbs_create(ctypes.byref(p), ctypes.c_void_p(stream), ctypes.byref(h)))
        self._h = h
        self._label = np.empty(self.window_size, np.int32)
        self._cid = np.empty(self.window_size, np.int32)

    # -- lifecycle
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.rtdbs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- host-buffer API
    def _host_points(self, pts, n: int) -> np.ndarray:
        a = np.ascontiguousarray(pts, dtype=np.float32)
        if a.shape != (n, self.dim):
            raise ValueError(f"expected points of shape ({n}, {self.dim}), got {a.shape}")
        return a

    def load_window(self, points) -> None:
        if isinstance(points, np.ndarray):
            a = self._host_points(points, self.window_size)
            _check(self._lib.rtdbs_load_window(self._h, a.ctypes.data, 0))
        else:  # device tensor
            _check(self._lib.rtdbs_load_window(self._h, _ptr(points), 1))

    def slide(self, new_points, label: Optional[np.ndarray] = None,
              cluster_id: Optional[np.ndarray] = None):
        """One slide; returns (label, cluster_id) host arrays (copies)."""
        a = self._host_points(new_points, self.stride_size)
        lab = self._label if label is None else label
        cid = self._cid if cluster_id is None else cluster_id
        _check(self._lib.rtdbs_slide(self._h, a.ctypes.data, lab.ctypes.data, cid.ctypes.data))
        if label is None:
            return lab.copy(), cid.copy()
        return lab, cid

    def slide_pipelined(self, new_points: np.ndarray, label: np.ndarray, cluster_id: np.ndarray) -> None:
        """One slide with host buffers, one slide in flight: returns once the
        previous pipelined slide is complete (its label/cluster_id arrays then
        hold its result); this call's arrays stay in use until the next
        pipelined call or sync().  Pinned arrays keep the copies asynchronous."""
        a = new_points
        if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous
                and a.shape == (self.stride_size, self.dim)):
            raise ValueError(f"expected contiguous float32 points of shape ({self.stride_size}, {self.dim})")
        for o in (label, cluster_id):
            if not (isinstance(o, np.ndarray) and o.dtype == np.int32 and o.flags.c_contiguous
                    and o.shape == (self.window_size,)):
                raise ValueError(f"expected contiguous int32 outputs of shape ({self.window_size},)")
        _check(self._lib.rtdbs_slide_pipelined(self._h, a.ctypes.data, label.ctypes.data, cluster_id.ctypes.data))

    def cluster(self):
        lab = np.empty(self.window_size, np.int32)
        cid = np.empty(self.window_size, np.int32)
        _check(self._lib.rtdbs_cluster(self._h, lab.ctypes.data, cid.ctypes.data, 0))
        return lab, cid

    def counts(self) -> np.ndarray:
        nn = np.empty(self.window_size, np.int32)
        _check(self._lib.rtdbs_get_counts(self._h, nn.ctypes.data, 0))
        return nn

    # -- device-buffer API
    def slide_async(self, d_new_points, d_label=None, d_cluster_id=None) -> None:
        _check(self._lib.rtdbs_slide_async(
            self._h, _ptr(d_new_points), 0 if d_label is None else _ptr(d_label),
            0 if d_cluster_id is None else _ptr(d_cluster_id)))

    def sync(self) -> None:
        _check(self._lib.rtdbs_sync(self._h))

    def device_outputs(self) -> Tuple[int, int]:
        lab, cid = ctypes.c_void_p(), ctypes.c_void_p()
        _check(self._lib.rtdbs_device_outputs(self._h, ctypes.byref(lab), ctypes.byref(cid)))
        return lab.value, cid.value

    def slide_profiled(self, d_new_points) -> dict:
        """One slide with per-phase CUDA-event timing (device input)."""
        t = PhaseTimes()
        _check(self._lib.rtdbs_slide_profiled(self._h, _ptr(d_new_points), ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in PhaseTimes._fields_}

    def stats(self) -> dict:
        s = Stats()
        _check(self._lib.rtdbs_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in Stats._fields_ if not f.startswith("reserved")}


def make_params(dim: int, window_size: int, stride_size: int, radius: float, min_pts: int,
                precision: str = "fp64", bbox: Optional[Tuple] = None, device: int = 0,
                use_graph: bool = True, cell_mult: int = 1, work_grab: int = 0,
                query_lanes: int = 0) -> Params:
    """rtdbs_params for one stream; cell_mult = grid cells per Eps (1 or 2),
    work_grab = work items per queue grab of the clustering warps (0: 8),
    query_lanes = lanes per query point in the count passes (0: 16 with one
    cell per Eps, 32 with two; 16 or 32)."""
    L = load_library()
    p = Params()
    _check(L.rtdbs_params_init(ctypes.byref(p)))
    p.dim, p.window, p.stride = int(dim), int(window_size), int(stride_size)
    p.min_pts, p.eps = int(min_pts), float(radius)
    p.precision = {"fp64": PREC_FP64, "fp32": PREC_FP32}[precision]
    p.device = int(device)
    p.flags = 0 if use_graph else FLAG_NO_GRAPH
    p.cell_mult = int(cell_mult)
    p.work_grab = int(work_grab)
    p.query_lanes = int(query_lanes)
    if bbox is not None:
        lo, hi = bbox
        p.has_bbox = 1
        for a in range(int(dim)):
            p.bbox_min[a] = float(lo[a])
            p.bbox_max[a] = float(hi[a])
    return p


def stream_bytes(params: Params) -> int:
    """Device bytes one stream occupies (a pool's admission cost); no GPU needed."""
    b = ctypes.c_int64()
    _check(load_library().rtdbs_stream_bytes(ctypes.byref(params), ctypes.byref(b)))
    return b.value


class Pool:
    """Many independent streams slid together, one launch per kernel phase."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, max_streams: int = 1024,
                 use_graph: bool = True, stream: int = 0):
        self._lib = load_library()
        pp = PoolParams()
        _check(self._lib.rtdbs_pool_params_init(ctypes.byref(pp)))
        pp.device, pp.max_streams = int(device), int(max_streams)
        pp.hbm_budget_bytes = int(hbm_budget_bytes)
        pp.flags = 0 if use_graph else FLAG_NO_GRAPH
        h = ctypes.c_void_p()
        _check(self._lib.rtdbs_pool_create(ctypes.byref(pp), ctypes.c_void_p(stream), ctypes.byref(h)))
        self._h = h
        self.windows = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.rtdbs_pool_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add_stream(self, params: Params) -> int:
        sid = ctypes.c_int32()
        _check(self._lib.rtdbs_pool_add_stream(self._h, ctypes.byref(params), ctypes.byref(sid)))
        self.windows[sid.value] = (params.window, params.stride, params.dim)
        return sid.value

    def remove_stream(self, sid: int) -> None:
        _check(self._lib.rtdbs_pool_remove_stream(self._h, int(sid)))
        self.windows.pop(sid, None)

    def load_window(self, sid: int, points) -> None:
        if isinstance(points, np.ndarray):
            a = np.ascontiguousarray(points, np.float32)
            _check(self._lib.rtdbs_pool_load_window(self._h, int(sid), a.ctypes.data, 0))
        else:
            _check(self._lib.rtdbs_pool_load_window(self._h, int(sid), _ptr(points), 1))

    def slide(self, sids, d_points) -> None:
        """One round: streams `sids` slide; d_points is a device tensor holding
        their new points back to back in that order."""
        ids = (ctypes.c_int32 * len(sids))(*[int(x) for x in sids])
        _check(self._lib.rtdbs_pool_slide(self._h, len(sids), ids, _ptr(d_points)))

    def slide_each(self, sids, d_points_each) -> None:
        """One round with each stream's new points in its own device buffer
        (a sequence of tensors or raw device addresses)."""
        n = len(sids)
        ids = (ctypes.c_int32 * n)(*[int(x) for x in sids])
        ptrs = (ctypes.c_void_p * n)(*[x if isinstance(x, int) else _ptr(x) for x in d_points_each])
        _check(self._lib.rtdbs_pool_slide_each(self._h, n, ids, ptrs))

    def sync(self) -> None:
        _check(self._lib.rtdbs_pool_sync(self._h))

    def slide_profiled(self, sids, d_points) -> dict:
        ids = (ctypes.c_int32 * len(sids))(*[int(x) for x in sids])
        t = PhaseTimes()
        _check(self._lib.rtdbs_pool_slide_profiled(self._h, len(sids), ids, _ptr(d_points), ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in PhaseTimes._fields_}

    def outputs(self, sid: int):
        W = self.windows[sid][0]
        lab = np.empty(W, np.int32)
        cid = np.empty(W, np.int32)
        _check(self._lib.rtdbs_pool_read_outputs(self._h, int(sid), lab.ctypes.data, cid.ctypes.data, 0))
        return lab, cid

    def counts(self, sid: int) -> np.ndarray:
        e = ctypes.c_void_p()
        _check(self._lib.rtdbs_pool_engine(self._h, int(sid), ctypes.byref(e)))
        nn = np.empty(self.windows[sid][0], np.int32)
        _check(self._lib.rtdbs_get_counts(e, nn.ctypes.data, 0))
        return nn

    def stats(self) -> dict:
        s = PoolStats()
        _check(self._lib.rtdbs_pool_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in PoolStats._fields_ if not f.startswith("reserved")}


FORMATS = {"auto": 0, "tao": 1, "geolife": 2, "rbf": 3, "eds": 4, "stock": 5}


def read_points(path: str, n_max: int, fmt: str = "auto"):
    """Reads a point file in one of the reference's formats.  Returns
    (points [n, dim] float32, bbox_min [dim], bbox_max [dim])."""
    xyz = np.zeros((max(int(n_max), 0), 3), np.float32)
    n = ctypes.c_int64()
    dim = ctypes.c_int32()
    lo = np.zeros(3, np.float32)
    hi = np.zeros(3, np.float32)
    _check(load_library().rtdbs_read_points(os.fsencode(path), FORMATS[fmt.lower()], int(n_max),
                                            xyz.ctypes.data, ctypes.byref(n), ctypes.byref(dim),
                                            lo.ctypes.data, hi.ctypes.data))
    d = dim.value
    return np.ascontiguousarray(xyz[: n.value, :d]), lo[:d].copy(), hi[:d].copy()
