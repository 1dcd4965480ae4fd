"""Seeded synthetic point streams with the shapes of the reference's workloads.

The reference's datasets (STK, RBF, TAO, GeoLife, EDS) are not distributed with
it, so every workload here is synthetic and seeded; the shapes, sizes and value
distributions follow the five benchmark configurations this engine is measured
on.  All coordinates are float32, row-major [n, dim].
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class StreamSpec:
    name: str
    dim: int
    window: int
    stride: int
    eps: float
    min_pts: int
    slides: int

    @property
    def n_total(self) -> int:
        return self.window + self.slides * self.stride


def gaussian_mixture(n: int, dim: int = 2, k: int = 20, box: float = 100.0, sigma: float = 1.0,
                     noise_frac: float = 0.10, seed: int = 0) -> np.ndarray:
    """k isotropic Gaussians (centres uniform in [0, box]^dim, std sigma) plus
    noise_frac uniform noise in [0, box]^dim, shuffled into stream order."""
    rng = np.random.default_rng(seed)
    n_noise = int(round(n * noise_frac))
    n_clu = n - n_noise
    centres = rng.uniform(0.0, box, size=(k, dim))
    which = rng.integers(0, k, size=n_clu)
    clu = centres[which] + rng.normal(0.0, sigma, size=(n_clu, dim))
    noise = rng.uniform(0.0, box, size=(n_noise, dim))
    pts = np.concatenate([clu, noise]).astype(np.float32)
    return pts[rng.permutation(n)]


def random_walkers(n_total: int, n_walkers: int = 2000, step: float = 1e-3,
                   start_box=(1.0, 1.0, 0.1), seed: int = 1) -> np.ndarray:
    """Trajectory-like 3-D stream: n_walkers random walkers started uniformly
    in a start_box, steps N(0, step) per axis, interleaved in time order
    (stream point t is walker t mod n_walkers at step t div n_walkers)."""
    rng = np.random.default_rng(seed)
    n_steps = -(-n_total // n_walkers)
    start = rng.uniform(0.0, 1.0, size=(n_walkers, 3)) * np.asarray(start_box)
    steps = rng.normal(0.0, step, size=(n_steps, n_walkers, 3))
    steps[0] = 0.0
    traj = start[None, :, :] + np.cumsum(steps, axis=0)
    return traj.reshape(-1, 3)[:n_total].astype(np.float32)


def offset_band_points(n: int, eps: float, partner_frac: float = 0.05, rel: float = 1e-6,
                       seed: int = 2) -> np.ndarray:
    """Precision workload: x~U[39.5,40.5], y~U[116,117], z~U[0,0.05] (a large
    common offset, GeoLife-like magnitudes) with partner_frac of the points
    placed at distance eps*(1 +- rel) from a random earlier anchor, so that many
    pairs sit inside the FP32 rounding band of eps^2."""
    rng = np.random.default_rng(seed)
    pts = np.empty((n, 3), np.float32)
    pts[:, 0] = rng.uniform(39.5, 40.5, n)
    pts[:, 1] = rng.uniform(116.0, 117.0, n)
    pts[:, 2] = rng.uniform(0.0, 0.05, n)
    n_part = int(round(n * partner_frac))
    idx = np.sort(rng.choice(np.arange(1, n), size=n_part, replace=False))
    anchor = np.maximum(idx - rng.integers(1, 2001, size=n_part), 0)
    # Partners are placed on the float32 grid itself: x and y are rounded
    # first, then z is solved in double for a squared distance of
    # (eps*(1 +- rel))^2 and the float32 z (within +-4 ulp) whose double
    # squared distance is closest to it is kept.  At these magnitudes the x/y
    # ulp (~4e-6) is far coarser than eps*rel, so without this the target
    # distance would be lost to rounding.
    target = (eps * (1.0 + rel * rng.choice([-1.0, 1.0], size=n_part))) ** 2
    a = pts[anchor].astype(np.float64)
    theta = rng.uniform(0.0, 2.0 * np.pi, n_part)
    frac_xy = rng.uniform(0.2, 0.8, n_part)
    rxy = np.sqrt(target * frac_xy)
    px = (a[:, 0] + rxy * np.cos(theta)).astype(np.float32).astype(np.float64)
    py = (a[:, 1] + rxy * np.sin(theta)).astype(np.float32).astype(np.float64)
    dz2 = target - (px - a[:, 0]) ** 2 - (py - a[:, 1]) ** 2
    dz = np.sqrt(np.maximum(dz2, 0.0)) * np.where(rng.random(n_part) < 0.5, -1.0, 1.0)
    z0 = (a[:, 2] + dz).astype(np.float32)
    best = z0.copy()
    best_err = np.full(n_part, np.inf)
    for k in range(-4, 5):
        zk = z0.copy()
        step = np.inf if k > 0 else -np.inf
        for _ in range(abs(k)):
            zk = np.nextafter(zk, np.float32(step))
        d2 = (px - a[:, 0]) ** 2 + (py - a[:, 1]) ** 2 + (zk.astype(np.float64) - a[:, 2]) ** 2
        err = np.abs(d2 - target)
        upd = err < best_err
        best[upd] = zk[upd]
        best_err[upd] = err[upd]
    pts[idx, 0] = px.astype(np.float32)
    pts[idx, 1] = py.astype(np.float32)
    pts[idx, 2] = best
    return pts


# The five benchmark configurations (sizes as measured; eps of the walker
# stream from seeded bisection on window 0 so that the mean FP64 neighbour
# count is ~20, see walker_eps()).
WALKER_EPS = 3.3328e-3

CFG0 = StreamSpec("mixture2d-W10k-S1k", dim=2, window=10_000, stride=1_000, eps=0.5, min_pts=5, slides=100)
CFG1 = StreamSpec("walkers3d-W1M-S10k", dim=3, window=1_000_000, stride=10_000, eps=WALKER_EPS,
                  min_pts=10, slides=200)
CFG2 = StreamSpec("offset3d-W500k-S5k", dim=3, window=500_000, stride=5_000, eps=1e-3, min_pts=8,
                  slides=20)


def cfg0_stream(seed: int = 0) -> np.ndarray:
    return gaussian_mixture(CFG0.n_total, dim=2, seed=seed)


def cfg1_stream(seed: int = 1, n_total: int | None = None) -> np.ndarray:
    return random_walkers(CFG1.n_total if n_total is None else n_total, seed=seed)


def cfg2_stream(seed: int = 2, n_total: int | None = None) -> np.ndarray:
    return offset_band_points(CFG2.n_total if n_total is None else n_total, CFG2.eps, seed=seed)


def mean_neighbours(window: np.ndarray, eps: float, n_query: int = 20000, seed: int = 0) -> float:
    """Mean neighbour count (self included) of a random sample of window points."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    tree = cKDTree(window.astype(np.float64))
    q = window[rng.choice(len(window), size=min(n_query, len(window)), replace=False)]
    return float(np.mean(tree.query_ball_point(q.astype(np.float64), r=eps, return_length=True)))


def walker_eps(target: float = 20.0, seed: int = 1, iters: int = 24) -> float:
    """Seeded bisection of eps on window 0 of the walker stream so that the
    mean neighbour count is `target` (how WALKER_EPS was obtained)."""
    win = cfg1_stream(seed=seed, n_total=CFG1.window)
    lo, hi = 1e-5, 1e-1
    for _ in range(iters):
        mid = float(np.sqrt(lo * hi))
        if mean_neighbours(win, mid) < target:
            lo = mid
        else:
            hi = mid
    return float(np.sqrt(lo * hi))


# ------------------------------------------------------------- stream mixes

@dataclass(frozen=True)
class MixStream:
    dim: int
    window: int
    stride: int
    eps: float
    min_pts: int
    seed: int
    box: float
    target: float = 0.0  # mean neighbour count the Eps was chosen for (0: not recorded)


def _divisor_near(W: int, target: int) -> int:
    """Divisor of W closest to target (at least 1)."""
    best = 1
    for d in range(1, int(np.sqrt(W)) + 1):
        if W % d == 0:
            for q in (d, W // d):
                if abs(q - target) < abs(best - target):
                    best = q
    return best


def mixed_streams(n: int = 256, seed: int = 3, w_lo: int = 1_000, w_hi: int = 200_000,
                  calibrate: bool = False) -> list:
    """Uneven independent streams: dim 2 or 3 (50/50), W log-uniform in
    [w_lo, w_hi], S a divisor of W near U[1%, 10%] of W, Gaussian-mixture data
    (20 Gaussians, sigma 1, 10% uniform noise) in a box scaled so densities
    differ per stream, Eps for a mean neighbour count drawn from U[10, 30],
    MinPts U[4, 16].  Eps starts from the density estimate of mix_eps; with
    `calibrate` it is then fitted to each stream's first window
    (calibrate_eps), as the benchmarks do."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dim = 2 if rng.random() < 0.5 else 3
        W = int(np.exp(rng.uniform(np.log(w_lo), np.log(w_hi))))
        W = max(w_lo, (W // 100) * 100)
        S = _divisor_near(W, int(W * rng.uniform(0.01, 0.10)))
        box = float(rng.uniform(40.0, 160.0))
        target = float(rng.uniform(10.0, 30.0))
        eps = mix_eps(W, dim, box, target)
        out.append(MixStream(dim, W, S, eps, int(rng.integers(4, 17)), 1000 + i, box, target))
    return [calibrate_eps(s) for s in out] if calibrate else out


def mix_eps(W: int, dim: int, box: float, target: float, k: int = 20, sigma: float = 1.0) -> float:
    """Eps giving about `target` neighbours for a mixture point: cluster
    points have density ~ n_c / (4 pi sigma^2)^(d/2) around them (a Gaussian
    seen from its own samples), n_c = 0.9 W / k."""
    n_c = 0.9 * W / k
    dens = n_c / (4.0 * np.pi * sigma * sigma) ** (dim / 2.0)
    vol = target / dens
    if dim == 2:
        return float(np.sqrt(vol / np.pi))
    return float((vol * 3.0 / (4.0 * np.pi)) ** (1.0 / 3.0))


def calibrate_eps(s: MixStream, n_query: int = 3000, tol: float = 0.01, max_evals: int = 8) -> MixStream:
    """The stream with Eps fitted so that the mean neighbour count (self
    included, FP64 distances) of a seeded sample of its first window is
    within `tol` of its target (clamped to [11, 29], leaving room for the
    sampling error: with 3,000 sampled points every stream of the 256-stream
    mix lands within 4% of its target over its whole window).  Secant steps on log(count)
    against log(Eps), starting from the density estimate."""
    from dataclasses import replace

    from scipy.spatial import cKDTree

    target = float(np.clip(s.target if s.target > 0 else 20.0, 11.0, 29.0))
    win = mix_points(s, s.window).astype(np.float64)
    tree = cKDTree(win, balanced_tree=False, compact_nodes=False)
    rng = np.random.default_rng(s.seed)
    q = win[rng.choice(len(win), size=min(n_query, len(win)), replace=False)]

    def mean(e: float) -> float:
        return float(np.mean(tree.query_ball_point(q, r=e, return_length=True)))

    e0 = s.eps
    m0 = mean(e0)
    e1 = e0 * (target / m0) ** (1.0 / s.dim)
    m1 = mean(e1)
    for _ in range(max_evals - 2):
        if abs(m1 - target) <= tol * target:
            break
        p = np.log(m1 / m0) / np.log(e1 / e0) if m1 != m0 and e1 != e0 else float(s.dim)
        p = float(np.clip(p, 0.5, 4.0))
        e0, m0 = e1, m1
        e1 = e1 * (target / m1) ** (1.0 / p)
        m1 = mean(e1)
    return replace(s, eps=float(e1))


def mix_points(s: MixStream, n_total: int, k: int = 20, block: int = 4096) -> np.ndarray:
    """The stream's first n_total points: k Gaussians (sigma 1, centres
    uniform in the box) with 10% uniform noise, drawn in blocks of `block`
    points from per-block seeds, so a stream's first points do not depend on
    how many are drawn (the window Eps is fitted on is the window the
    benchmarks slide from)."""
    centres = np.random.default_rng(s.seed).uniform(0.0, s.box, size=(k, s.dim))
    out = np.empty((-(-n_total // block) * block, s.dim), np.float64)
    for b in range(len(out) // block):
        r = np.random.default_rng([s.seed, b])
        blk = centres[r.integers(0, k, size=block)] + r.normal(0.0, 1.0, size=(block, s.dim))
        noise = r.random(block) < 0.10
        blk[noise] = r.uniform(0.0, s.box, size=(int(noise.sum()), s.dim))
        out[b * block:(b + 1) * block] = blk
    return out[:n_total].astype(np.float32)
