"""Generate the golden fixtures in this directory from the reference itself.

Every expected output here comes from the reference's own CPU checker,
cluster_with_cpu (src/dbscan/util.cpp:299-354), compiled from the reference's
unmodified sources by oracle/Makefile into oracle/_ref/libref_cpu.so.  Inputs
are seeded synthetic windows and streams (rtdbstream_gb300.workloads).

Run from the repository root where the reference tree is available:
    python tests/golden/make_golden.py
Each fixture is an .npz with: pts [n, dim] float32, eps, min_pts, and either
one window (nn, label, cid: [W]) or a stream (W, S, nn/label/cid: [slides, W],
slot-indexed as the reference's ring buffer).  Noise ids are normalised to the
point's own slot (the reference leaves them untouched).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from rtdbstream_gb300 import workloads as wl  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def save_window(name: str, pts: np.ndarray, eps: float, min_pts: int) -> None:
    nn, lab, cid = oracle.window_reference(pts, eps, min_pts)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), pts=pts.astype(np.float32),
                        eps=np.float64(eps), min_pts=np.int32(min_pts), nn=nn, label=lab, cid=cid)
    print(f"{name}: n={len(pts)} dim={pts.shape[1]} labels={np.bincount(lab, minlength=3).tolist()}")


def save_stream(name: str, stream: np.ndarray, W: int, S: int, slides: int, eps: float,
                min_pts: int) -> None:
    stream = stream[: W + slides * S].astype(np.float32)
    nn = np.empty((slides, W), np.int32)
    lab = np.empty((slides, W), np.int32)
    cid = np.empty((slides, W), np.int32)
    for k in range(1, slides + 1):
        win = oracle.window_of(stream, W, S, k)
        nn[k - 1], lab[k - 1], cid[k - 1] = oracle.window_reference(win, eps, min_pts)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), pts=stream, eps=np.float64(eps),
                        min_pts=np.int32(min_pts), W=np.int32(W), S=np.int32(S), nn=nn, label=lab,
                        cid=cid)
    print(f"{name}: W={W} S={S} slides={slides} labels={np.bincount(lab.ravel(), minlength=3).tolist()}")


def main() -> None:
    oracle.build(ref=True)
    if oracle.ref_lib() is None:
        raise SystemExit("reference CPU library unavailable: the reference tree is needed")
    rng = np.random.default_rng(2024)

    save_window("mix2d_w2000", wl.gaussian_mixture(2000, dim=2, k=8, box=25.0, seed=11), 0.5, 5)
    save_window("mix3d_w2000", wl.gaussian_mixture(2000, dim=3, k=8, box=20.0, seed=12), 1.3, 6)
    save_window("stk1d_w2000", wl.gaussian_mixture(2000, dim=1, k=6, box=10.0, sigma=0.3, seed=13),
                0.07, 2)
    save_window("walkers3d_w3000", wl.random_walkers(3000, n_walkers=60, step=1e-3, seed=14),
                3.3e-3, 10)
    save_window("band3d_w3000", wl.offset_band_points(3000, 1e-3, partner_frac=0.3, seed=15), 1e-3, 2)
    dup = np.concatenate([np.repeat(rng.uniform(0, 10, (5, 2)), 60, axis=0),
                          rng.uniform(0, 10, (200, 2))]).astype(np.float32)
    save_window("dup2d_w500", dup[rng.permutation(len(dup))], 0.25, 4)
    save_window("noise2d_w1000", rng.uniform(0, 1000, (1000, 2)).astype(np.float32), 0.5, 3)
    save_window("ball3d_w800", rng.normal(0, 0.01, (800, 3)).astype(np.float32), 0.5, 20)
    save_window("edge2d_w64", np.array([[0, 0], [0.5, 0], [1.0, 0], [1.5, 0], [0.25, 0.25],
                                        [3, 3], [3, 3.5], [3.5, 3], [10, 10]] * 7 + [[20, 20]],
                                       np.float32), 0.5, 3)

    save_stream("stream_mix2d_W1000_S250", wl.gaussian_mixture(1000 + 8 * 250, dim=2, k=6, box=20.0,
                                                                seed=21), 1000, 250, 8, 0.5, 5)
    save_stream("stream_walk3d_W1200_S400",
                wl.random_walkers(1200 + 6 * 400, n_walkers=40, step=1e-3, seed=22), 1200, 400, 6,
                3.3e-3, 8)
    save_stream("stream_band3d_W1500_S500",
                wl.offset_band_points(1500 + 5 * 500, 1e-3, partner_frac=0.3, seed=23), 1500, 500, 5,
                1e-3, 2)
    save_stream("stream_mix2d_W600_S600", wl.gaussian_mixture(600 * 5, dim=2, k=5, box=15.0, seed=24),
                600, 600, 4, 0.5, 5)


if __name__ == "__main__":
    main()
