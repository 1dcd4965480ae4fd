"""Long streams: the engine, called through the C ABI, compared bit-exactly
with the CPU oracle on every slide over several full turnovers of the window
(so every slot has been refilled several times, the expired chunks' kept
order is in use and the previous clustering is reused across many slides),
and the reference's debug counters (src/dbscan/dbscan.cpp:145-212) checked
for consistency.

The reference re-clusters every window from scratch
(src/dbscan/dbscan.cpp:2314-2336); these tests hold the reusing path to that
result.
"""
import numpy as np
import pytest

import oracle as O
from rtdbstream_gb300 import Engine
from rtdbstream_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build(ref=False)
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def run(pts, W, S, eps, mp, slides, precision="fp64", cell_mult=1, query_lanes=0, use_graph=True):
    eng = Engine(pts.shape[1], W, S, eps, mp, precision=precision, cell_mult=cell_mult,
                 query_lanes=query_lanes, use_graph=use_graph)
    eng.load_window(pts[:W])
    out, stats = [], []
    for k in range(slides):
        lab, cid = eng.slide(pts[W + k * S: W + (k + 1) * S])
        out.append((eng.counts(), lab, cid))
        stats.append(eng.stats())
    eng.close()
    return out, stats


def check(pts, W, S, eps, mp, slides, precision, what, **kw):
    got, stats = run(pts, W, S, eps, mp, slides, precision=precision, **kw)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    enn, elab, ecid = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=slides)
    for k, (nn, lab, cid) in enumerate(got):
        assert np.array_equal(nn, enn[k]), f"{what}: counts differ on slide {k + 1}"
        assert np.array_equal(lab, elab[k]), f"{what}: labels differ on slide {k + 1}"
        assert np.array_equal(cid, ecid[k]), f"{what}: ids differ on slide {k + 1}"
    return stats, elab


def test_walkers_three_turnovers():
    """Trajectory stream: components lose their oldest cores every slide and
    rarely fall apart, so part of the previous clustering is kept."""
    W, S, slides = 20_000, 1_000, 60
    pts = wl.random_walkers(W + slides * S, n_walkers=40, seed=31)
    stats, elab = check(pts, W, S, 3.3e-3, 10, slides, "fp64", "walkers")
    assert max(st["reused_cores"] for st in stats[W // S:]) > 0
    last = stats[-1]
    assert last["cluster_hits"] > 0 and last["query_hits"] > 0
    assert last["query_hits"] <= last["query_tests"] and last["cluster_hits"] <= last["cluster_tests"]
    assert last["dist_tests"] == last["query_tests"] + last["cluster_tests"]
    assert 0 < last["max_query_tests"] <= last["query_tests"]
    # counters are cumulative
    assert all(b["query_tests"] >= a["query_tests"] for a, b in zip(stats, stats[1:]))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("cell_mult", [1, 2])
def test_mixture_turnovers(precision, cell_mult):
    """Shuffled Gaussian mixture: expiry is spread over every cluster, so
    nearly every component is damaged on every slide."""
    W, S, slides = 6_000, 600, 32
    pts = wl.gaussian_mixture(W + slides * S, dim=2, k=6, box=30.0, seed=32)
    check(pts, W, S, 0.45, 6, slides, precision, f"mix/{precision}/K{cell_mult}", cell_mult=cell_mult)


def test_mixture_3d_full_warp_queries():
    W, S, slides = 9_000, 450, 44
    pts = wl.gaussian_mixture(W + slides * S, dim=3, k=8, box=20.0, seed=33)
    check(pts, W, S, 0.8, 8, slides, "fp64", "mix3d/q32", query_lanes=32)


def test_small_minpts_and_direct_launches():
    """MinPts 2 (every point with a neighbour is core) and 3, kernels
    launched directly instead of a graph replay."""
    W, S, slides = 5_000, 250, 44
    pts = wl.gaussian_mixture(W + slides * S, dim=2, k=10, box=60.0, seed=34)
    for mp in (2, 3):
        check(pts, W, S, 0.5, mp, slides, "fp64", f"mp{mp}", use_graph=False)


def test_precision_band_stream():
    """Pairs at Eps (1 +- 1e-6): the FP64 re-check decides the clustering's
    edges as well as the counts."""
    W, S, slides = 12_000, 1_200, 24
    pts = wl.offset_band_points(W + slides * S, 1e-3, partner_frac=0.3, seed=35)
    check(pts, W, S, 1e-3, 2, slides, "fp64", "band")


def test_cluster_without_slide_keeps_result():
    """rtdbs_cluster between slides re-derives the same clustering (nothing
    new arrived), and sliding on afterwards stays exact."""
    W, S = 4_000, 400
    pts = wl.random_walkers(W + 30 * S, n_walkers=16, seed=36)
    eps, mp = 3.3e-3, 6
    eng = Engine(3, W, S, eps, mp)
    eng.load_window(pts[:W])
    enn, elab, ecid = O.stream(pts, W, S, eps, mp, O.MODE_FP64, first_slide=1, n_out=30)
    for k in range(30):
        lab, cid = eng.slide(pts[W + k * S: W + (k + 1) * S])
        assert np.array_equal(lab, elab[k]) and np.array_equal(cid, ecid[k]), f"slide {k + 1}"
        if k % 7 == 3:
            lab2, cid2 = eng.cluster()
            assert np.array_equal(lab2, elab[k]) and np.array_equal(cid2, ecid[k]), f"cluster after {k + 1}"
    eng.close()
