"""CPU oracle for the per-slide streaming DBSCAN path -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline legs
import this package.  It is the checker, never the product: the package
``rtdbstream_gb300`` has no code path that reaches it.

* ``liboracle.so`` (``rtdbs_oracle.c``): our C restatement of the reference
  algorithm -- a brute-force restatement of ``cluster_with_cpu``
  (src/dbscan/util.cpp:299-354) and a grid DBSCAN with FP32 (reference) and
  FP64 neighbour predicates.
* ``_ref/libref_cpu.so``: the reference's own ``src/dbscan/util.cpp`` compiled
  from its sources by ``oracle/Makefile`` (only where the reference tree is
  present; it pins the restatement and generated ``tests/golden``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_cpu.so")

def reference_tree() -> Optional[str]:
    """Where the reference's sources lie: $RTDBS_REFERENCE_TREE, else the
    location the build recipe (oracle/Makefile) reads them from; None where
    they are absent (the GPU machine has only this package's restatement)."""
    tree = os.environ.get("RTDBS_REFERENCE_TREE")
    if not tree:
        r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
        tree = r.stdout.strip()
    return tree if tree and os.path.isdir(os.path.join(tree, "src", "dbscan")) else None


MODE_FP64 = 0
MODE_FP32 = 1


class OracleStats(ctypes.Structure):
    _fields_ = [("dist_tests", ctypes.c_int64), ("band_pairs", ctypes.c_int64),
                ("cells", ctypes.c_int64)]


def build(ref: bool = True) -> None:
    """Compile liboracle.so (always) and the reference CPU library (when the
    reference's sources are present on this machine; otherwise says so)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if not ref:
        return
    tree = reference_tree()
    if tree:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={tree}"], check=True)
    else:
        print("oracle: reference sources not present here; only the restatement is built")


_lib = None
_ref = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_window_grid.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p,
                                         ctypes.POINTER(OracleStats)]
        L.oracle_window_bruteforce_ref.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_int, _i32p, _i32p, _i32p]
        L.oracle_stream.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p,
                                    ctypes.c_void_p]
        L.oracle_band.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_float),
                                  ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own cluster_with_cpu, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB_PATH):
        L = ctypes.CDLL(REF_LIB_PATH)
        L.ref_cluster_with_cpu.argtypes = [_f32p, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                           _i32p, _i32p, _i32p]
        _ref = L
    return _ref


def _pts(pts: np.ndarray) -> tuple[np.ndarray, int, int]:
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    if pts.ndim != 2 or not 1 <= pts.shape[1] <= 3:
        raise ValueError("points must be [n, dim] with dim in 1..3")
    return pts, pts.shape[0], pts.shape[1]


def window_grid(pts, eps: float, min_pts: int, mode: int = MODE_FP64):
    """Grid DBSCAN of one window -> (nn, label, cid, stats)."""
    pts, n, dim = _pts(pts)
    nn = np.empty(n, np.int32); lab = np.empty(n, np.int32); cid = np.empty(n, np.int32)
    st = OracleStats()
    rc = lib().oracle_window_grid(pts, n, dim, float(eps), int(min_pts), int(mode), nn, lab, cid,
                                  ctypes.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle_window_grid failed ({rc})")
    return nn, lab, cid, {"dist_tests": st.dist_tests, "band_pairs": st.band_pairs, "cells": st.cells}


def window_bruteforce(pts, eps: float, min_pts: int):
    """Restated cluster_with_cpu (FP32, O(n^2)) -> (nn, label, cid)."""
    pts, n, dim = _pts(pts)
    nn = np.empty(n, np.int32); lab = np.empty(n, np.int32); cid = np.empty(n, np.int32)
    rc = lib().oracle_window_bruteforce_ref(pts, n, dim, float(eps), int(min_pts), nn, lab, cid)
    if rc != 0:
        raise RuntimeError(f"oracle_window_bruteforce_ref failed ({rc})")
    return nn, lab, cid


def window_reference(pts, eps: float, min_pts: int):
    """The reference's own cluster_with_cpu on one window -> (nn, label, cid).
    Noise ids are normalised to the point's own slot (the reference leaves
    them untouched).  Raises if the reference library was not built here."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference CPU library not built (needs the reference tree)")
    pts, n, dim = _pts(pts)
    xyz = np.zeros((n, 3), np.float32)
    xyz[:, :dim] = pts
    nn = np.zeros(n, np.int32); lab = np.zeros(n, np.int32)
    cid = np.arange(n, dtype=np.int32)
    rc = L.ref_cluster_with_cpu(np.ascontiguousarray(xyz), n, ctypes.c_float(np.float32(eps)),
                                int(min_pts), nn, lab, cid)
    if rc != 0:
        raise RuntimeError(f"ref_cluster_with_cpu failed ({rc})")
    cid = np.where(lab == 2, np.arange(n, dtype=np.int32), cid).astype(np.int32)
    return nn, lab, cid


def stream(points, W: int, S: int, eps: float, min_pts: int, mode: int = MODE_FP64,
           first_slide: int = 1, n_out: Optional[int] = None, bruteforce: bool = False):
    """Sliding-window oracle.  Returns (nn, label, cid) each [n_out, W],
    indexed by ring slot, for slides first_slide .. first_slide+n_out-1."""
    pts, n_total, dim = _pts(points)
    if n_out is None:
        n_out = (n_total - W) // S - first_slide + 1
    nn = np.empty((n_out, W), np.int32); lab = np.empty((n_out, W), np.int32)
    cid = np.empty((n_out, W), np.int32)
    rc = lib().oracle_stream(pts, n_total, dim, W, S, float(eps), int(min_pts), int(mode),
                             1 if bruteforce else 0, int(first_slide), int(n_out), nn, lab, cid, None)
    if rc != 0:
        raise RuntimeError(f"oracle_stream failed ({rc})")
    return nn, lab, cid


def band(eps: float):
    lo = ctypes.c_float(); hi = ctypes.c_float(); ok = ctypes.c_int()
    lib().oracle_band(float(eps), ctypes.byref(lo), ctypes.byref(hi), ctypes.byref(ok))
    return lo.value, hi.value, bool(ok.value)


def window_of(points: np.ndarray, W: int, S: int, slide: int) -> np.ndarray:
    """Window contents after `slide` slides, in ring-slot order."""
    pts = np.asarray(points, np.float32)
    t = np.arange(slide * S, slide * S + W)
    win = np.empty((W, pts.shape[1]), np.float32)
    win[t % W] = pts[t]
    return win
