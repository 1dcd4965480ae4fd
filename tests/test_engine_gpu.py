"""GPU parity of the engine, called through the C ABI, against the CPU oracle
and against fixtures produced by the reference's own cluster_with_cpu.

Integer results are compared bit-exactly: neighbour counts, labels and
cluster ids (noise ids are the point's own slot by definition).
"""
import os

import numpy as np
import pytest

from conftest import golden_files, load_golden

import oracle as O
from rtdbstream_gb300 import Engine, RtdbsError
from rtdbstream_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build(ref=False)
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def run_stream(points, W, S, eps, mp, n_slides, precision="fp64", use_graph=True, bbox=None, cell_mult=1,
               query_lanes=0):
    eng = Engine(points.shape[1], W, S, eps, mp, precision=precision, use_graph=use_graph, bbox=bbox,
                 cell_mult=cell_mult, query_lanes=query_lanes)
    eng.load_window(points[:W])
    labs, cids, nns = [], [], []
    for k in range(n_slides):
        lab, cid = eng.slide(points[W + k * S: W + (k + 1) * S])
        labs.append(lab)
        cids.append(cid)
        nns.append(eng.counts())
    st = eng.stats()
    eng.close()
    return np.array(nns), np.array(labs), np.array(cids), st


def assert_same(got, exp, what=""):
    nn, lab, cid = got
    enn, elab, ecid = exp
    assert np.array_equal(nn, enn), f"{what}: counts differ at {np.argwhere(nn != enn)[:5].tolist()}"
    assert np.array_equal(lab, elab), f"{what}: labels differ at {np.argwhere(lab != elab)[:5].tolist()}"
    keep = elab != 2
    assert np.array_equal(cid[keep], ecid[keep]), f"{what}: ids differ"
    assert np.array_equal(np.where(lab == 2, cid, -1),
                          np.where(lab == 2, np.broadcast_to(np.arange(lab.shape[-1]), lab.shape), -1))


@pytest.mark.parametrize("path", golden_files("window"), ids=os.path.basename)
def test_window_fp32_matches_reference_golden(path):
    g = load_golden(path)
    pts = g["pts"]
    W = len(pts)
    eng = Engine(pts.shape[1], W, W, float(g["eps"]), int(g["min_pts"]), precision="fp32")
    eng.load_window(pts)
    lab, cid = eng.cluster()
    nn = eng.counts()
    eng.close()
    assert_same((nn, lab, cid), (g["nn"], g["label"], g["cid"]), os.path.basename(path))


@pytest.mark.parametrize("path", golden_files("stream"), ids=os.path.basename)
def test_stream_fp32_matches_reference_golden(path):
    g = load_golden(path)
    W, S = int(g["W"]), int(g["S"])
    slides = g["nn"].shape[0]
    got = run_stream(g["pts"], W, S, float(g["eps"]), int(g["min_pts"]), slides, precision="fp32")
    assert_same(got[:3], (g["nn"], g["label"], g["cid"]), os.path.basename(path))


@pytest.mark.parametrize("path", golden_files("stream"), ids=os.path.basename)
def test_stream_fp64_matches_oracle(path):
    g = load_golden(path)
    W, S = int(g["W"]), int(g["S"])
    slides = g["nn"].shape[0]
    eps, mp = float(g["eps"]), int(g["min_pts"])
    got = run_stream(g["pts"], W, S, eps, mp, slides, precision="fp64")
    exp = O.stream(g["pts"], W, S, eps, mp, O.MODE_FP64, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, os.path.basename(path))


CASES = [
    # name, points, W, S, eps, min_pts, slides
    ("mix2d_W10k_S1k", lambda: wl.gaussian_mixture(10_000 + 6 * 1_000, dim=2, seed=3), 10_000, 1_000, 0.5, 5, 6),
    ("walk3d_W60k_S6k", lambda: wl.random_walkers(60_000 + 4 * 6_000, n_walkers=300, seed=4), 60_000, 6_000,
     3.3e-3, 10, 4),
    ("band3d_W20k_S2k", lambda: wl.offset_band_points(20_000 + 4 * 2_000, 1e-3, partner_frac=0.3, seed=5),
     20_000, 2_000, 1e-3, 2, 4),
    ("stk1d_W8k_S2k", lambda: wl.gaussian_mixture(8_000 + 3 * 2_000, dim=1, k=6, box=10.0, sigma=0.3, seed=6),
     8_000, 2_000, 0.01, 4, 3),
    ("big_stride_W40k_S20k", lambda: wl.gaussian_mixture(40_000 + 3 * 20_000, dim=2, k=30, box=100.0, seed=7),
     40_000, 20_000, 0.4, 6, 3),
    ("S_eq_W_3d", lambda: wl.gaussian_mixture(3_000 * 4, dim=3, k=6, box=15.0, seed=8), 3_000, 3_000, 1.0, 5, 3),
    # MinPts 32: the longest neighbour lists kept (30 entries)
    ("mix3d_mp32_W12k", lambda: wl.gaussian_mixture(12_000 + 4 * 1_200, dim=3, k=10, box=30.0, seed=11),
     12_000, 1_200, 0.9, 32, 4),
    # MinPts 40: no lists, the label pass scans the grid
    ("mix2d_mp40_W8k", lambda: wl.gaussian_mixture(8_000 + 4 * 800, dim=2, k=8, box=30.0, seed=12),
     8_000, 800, 0.6, 40, 4),
]


@pytest.mark.parametrize("name,gen,W,S,eps,mp,slides", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_streams_match_oracle(name, gen, W, S, eps, mp, slides, precision):
    pts = gen()
    got = run_stream(pts, W, S, eps, mp, slides, precision=precision)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    exp = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, f"{name}/{precision}")
    assert got[3]["dist_tests"] > 0 and got[3]["slides"] == slides
    if name.startswith("band") and precision == "fp64":
        assert got[3]["band_rechecks"] > 0
        # the FP64 relation really differs from the reference's FP32 one here
        e32 = O.stream(pts, W, S, eps, mp, O.MODE_FP32, first_slide=1, n_out=slides)
        assert not np.array_equal(exp[0], e32[0])


def test_graph_and_direct_launch_identical():
    pts = wl.gaussian_mixture(5_000 + 5 * 500, dim=2, k=10, box=40.0, seed=9)
    a = run_stream(pts, 5_000, 500, 0.5, 5, 5, use_graph=True)
    b = run_stream(pts, 5_000, 500, 0.5, 5, 5, use_graph=False)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


def test_bbox_given_equals_bbox_from_first_window():
    pts = wl.gaussian_mixture(4_000 + 4 * 1_000, dim=2, k=8, box=30.0, seed=10)
    bbox = (pts.min(axis=0), pts.max(axis=0))
    a = run_stream(pts, 4_000, 1_000, 0.5, 5, 4, bbox=bbox)
    b = run_stream(pts, 4_000, 1_000, 0.5, 5, 4)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


def test_points_outside_bbox_are_exact():
    """A stream that drifts far outside the given box is clamped into
    boundary cells and must still be exact."""
    pts = wl.gaussian_mixture(3_000 + 3 * 1_000, dim=2, k=6, box=20.0, seed=11)
    pts[3_000:] += np.float32(50.0)
    bbox = ((0.0, 0.0), (20.0, 20.0))
    got = run_stream(pts, 3_000, 1_000, 0.5, 4, 3, bbox=bbox)
    exp = O.stream(pts, 3_000, 1_000, 0.5, 4, O.MODE_FP64, first_slide=1, n_out=3)
    assert_same(got[:3], exp, "drift")


def test_duplicates_and_nonfinite_points():
    rng = np.random.default_rng(12)
    base = np.repeat(rng.uniform(0, 5, (20, 2)), 40, axis=0).astype(np.float32)
    pts = np.concatenate([base, rng.uniform(0, 5, (400, 2)).astype(np.float32)])
    pts = pts[rng.permutation(len(pts))]
    pts[7] = np.nan
    pts[11] = np.inf
    W, S = 800, 200
    got = run_stream(pts, W, S, 0.3, 4, 2)
    exp = O.stream(pts, W, S, 0.3, 4, O.MODE_FP64, first_slide=1, n_out=2)
    assert_same(got[:3], exp, "dups/nonfinite")


def test_determinism_repeated_runs():
    pts = wl.random_walkers(30_000 + 3 * 3_000, n_walkers=200, seed=13)
    a = run_stream(pts, 30_000, 3_000, 3.3e-3, 8, 3)
    b = run_stream(pts, 30_000, 3_000, 3.3e-3, 8, 3)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


def test_slide_async_device_buffers():
    torch = pytest.importorskip("torch")
    pts = wl.gaussian_mixture(6_000 + 3 * 2_000, dim=2, k=10, box=40.0, seed=14)
    W, S = 6_000, 2_000
    eng = Engine(2, W, S, 0.5, 5)
    dev = torch.from_numpy(pts).cuda()
    eng.load_window(dev[:W].contiguous())
    lab = torch.empty(W, dtype=torch.int32, device="cuda")
    cid = torch.empty(W, dtype=torch.int32, device="cuda")
    exp = O.stream(pts, W, S, 0.5, 5, O.MODE_FP64, first_slide=1, n_out=3)
    for k in range(3):
        eng.slide_async(dev[W + k * S: W + (k + 1) * S].contiguous(), lab, cid)
        eng.sync()
        assert np.array_equal(lab.cpu().numpy(), exp[1][k])
        keep = exp[1][k] != 2
        assert np.array_equal(cid.cpu().numpy()[keep], exp[2][k][keep])
    eng.close()


def test_slide_pipelined_host_buffers():
    """One slide in flight: each call returns the previous slide's result into
    that call's (pinned) buffers; the last one arrives with sync()."""
    torch = pytest.importorskip("torch")
    W, S, n = 8_000, 1_000, 6
    pts = wl.gaussian_mixture(W + n * S, dim=3, k=8, box=20.0, seed=21)
    exp = O.stream(pts, W, S, 0.8, 6, O.MODE_FP64, first_slide=1, n_out=n)
    pin = lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory().numpy()
    h_in = pin((W + n * S, 3), torch.float32)
    h_in[:] = pts
    outs = [(pin(W, torch.int32), pin(W, torch.int32)) for _ in range(n)]
    with Engine(3, W, S, 0.8, 6) as eng:
        eng.load_window(h_in[:W])
        for k in range(n):
            eng.slide_pipelined(h_in[W + k * S: W + (k + 1) * S], *outs[k])
            if k:  # the previous slide is complete
                lab, cid = outs[k - 1]
                assert np.array_equal(lab, exp[1][k - 1]), k - 1
                keep = exp[1][k - 1] != 2
                assert np.array_equal(cid[keep], exp[2][k - 1][keep]), k - 1
        eng.sync()
        lab, cid = outs[n - 1]
        assert np.array_equal(lab, exp[1][n - 1])
        assert np.array_equal(cid[exp[1][n - 1] != 2], exp[2][n - 1][exp[1][n - 1] != 2])
        assert np.array_equal(eng.counts(), exp[0][n - 1])


def test_slide_pipelined_mixed_with_other_calls():
    """Pipelined slides interleaved with device-buffer slides, counts and a
    re-cluster: every result matches the oracle (the pipelined slide's
    output copies finish before any later call rewrites the labels)."""
    torch = pytest.importorskip("torch")
    W, S, n = 6_000, 1_500, 7
    pts = wl.gaussian_mixture(W + n * S, dim=2, k=6, box=25.0, seed=23)
    exp = O.stream(pts, W, S, 0.6, 5, O.MODE_FP64, first_slide=1, n_out=n)
    pin = lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory().numpy()
    outs = [(pin(W, torch.int32), pin(W, torch.int32)) for _ in range(n)]
    dev = torch.from_numpy(pts).cuda()
    d_lab = torch.empty(W, dtype=torch.int32, device="cuda")
    d_cid = torch.empty(W, dtype=torch.int32, device="cuda")

    def same(lab, cid, k):
        keep = exp[1][k] != 2
        return np.array_equal(lab, exp[1][k]) and np.array_equal(cid[keep], exp[2][k][keep])

    with Engine(2, W, S, 0.6, 5) as eng:
        eng.load_window(pts[:W])
        new = lambda k: np.ascontiguousarray(pts[W + k * S: W + (k + 1) * S])
        eng.slide_pipelined(new(0), *outs[0])
        eng.slide_pipelined(new(1), *outs[1])
        assert same(*outs[0], 0)
        # a device-buffer slide while slide 1's copies may still run
        eng.slide_async(dev[W + 2 * S: W + 3 * S].contiguous(), d_lab, d_cid)
        eng.sync()
        assert same(*outs[1], 1)
        assert same(d_lab.cpu().numpy(), d_cid.cpu().numpy(), 2)
        eng.slide_pipelined(new(3), *outs[3])
        assert np.array_equal(eng.counts(), exp[0][3])  # synchronising: slide 3 is complete
        assert same(*outs[3], 3)
        lab, cid = eng.cluster()  # the window as it stands: slide 3's clustering again
        assert same(lab, cid, 3)
        eng.slide_pipelined(new(4), *outs[4])
        lab, cid = eng.slide(new(5))  # synchronous slide after a pipelined one
        assert same(*outs[4], 4) and same(lab, cid, 5)
        eng.slide_pipelined(new(6), *outs[6])
        eng.sync()
        assert same(*outs[6], 6)


def test_cluster_twice_without_slide():
    pts = wl.gaussian_mixture(4_000 + 1_000, dim=3, k=6, box=15.0, seed=15)
    with Engine(3, 4_000, 1_000, 1.0, 5) as eng:
        eng.load_window(pts[:4_000])
        a = eng.cluster()
        b = eng.cluster()
        c = eng.slide(pts[4_000:])
        d = eng.cluster()
    exp0 = O.window_grid(pts[:4_000], 1.0, 5, O.MODE_FP64)
    exp1 = O.window_grid(O.window_of(pts, 4_000, 1_000, 1), 1.0, 5, O.MODE_FP64)
    for (lab, cid), (_, elab, ecid, _) in ((a, exp0), (b, exp0), (c, exp1), (d, exp1)):
        assert np.array_equal(lab, elab) and np.array_equal(cid, ecid)


def test_api_errors():
    with pytest.raises(RtdbsError) as ei:
        Engine(2, 100, 30, 0.5, 4)
    assert ei.value.status == -1
    eng = Engine(2, 100, 20, 0.5, 4)
    with pytest.raises(RtdbsError) as ei:
        eng.slide(np.zeros((20, 2), np.float32))
    assert ei.value.status == -4
    eng.close()


def test_walkers_full_window_exact():
    """The 1M-point walker window (the benchmark workload), two slides,
    compared bit-exactly with the FP64 oracle."""
    spec = wl.CFG1
    pts = wl.cfg1_stream(n_total=spec.window + 2 * spec.stride)
    got = run_stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, 2)
    exp = O.stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, O.MODE_FP64, first_slide=1, n_out=2)
    assert_same(got[:3], exp, "walkers 1M")


def test_precision_config_full_size():
    """The precision configuration at full size (W = 500k, S = 5k, large
    common offset, 5% of points at Eps(1 +- 1e-6) from an anchor): labels,
    ids and counts equal the FP64 oracle, FP64 re-checks happen, and the
    FP64 relation really differs from the reference's FP32 one here."""
    spec = wl.CFG2
    pts = wl.cfg2_stream(n_total=spec.window + 3 * spec.stride)
    got = run_stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, 3)
    exp = O.stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, O.MODE_FP64, first_slide=1, n_out=3)
    assert_same(got[:3], exp, "offset 500k")
    assert got[3]["band_rechecks"] > 0
    e32 = O.stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, O.MODE_FP32, first_slide=1, n_out=3)
    assert not np.array_equal(exp[0], e32[0])


def test_mixture_config_all_slides():
    """The 2-D mixture configuration as specified: W = 10k, S = 1k, all 100
    slides, every window equal to the FP64 oracle and, in FP32 mode, to the
    reference semantics."""
    spec = wl.CFG0
    pts = wl.cfg0_stream()
    for precision, mode in (("fp64", O.MODE_FP64), ("fp32", O.MODE_FP32)):
        got = run_stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, spec.slides, precision=precision)
        exp = O.stream(pts, spec.window, spec.stride, spec.eps, spec.min_pts, mode, first_slide=1,
                       n_out=spec.slides)
        assert_same(got[:3], exp, f"mixture W10k/{precision}")


def reuse_stream(seed=21):
    """A window whose oldest points are far-away noise and a bridge between
    two blobs, its newest points three stationary 2-D blobs: the first slides
    expire only noise and bridge points, so blob components lose no core
    (reused) while the bridged pair splits; new points land next to one blob
    (insertions into a kept component) and in the noise region."""
    rng = np.random.default_rng(seed)
    W, S = 6_000, 500
    noise = rng.uniform(50.0, 60.0, size=(1_500, 2))
    bridge = np.stack([np.linspace(0.5, 9.5, 500), np.full(500, 0.0)], axis=1) + rng.normal(0, 0.01, (500, 2))
    blobs = np.concatenate([rng.normal(c, 0.4, size=(1_334, 2)) for c in ((0.0, 0.0), (10.0, 0.0), (0.0, 10.0))])
    blobs = blobs[rng.permutation(len(blobs))][: W - 2_000]
    window = np.concatenate([noise, bridge, blobs])
    new = np.concatenate([np.concatenate([rng.normal((0.0, 10.0), 0.4, size=(100, 2)),
                                          rng.uniform(50.0, 60.0, size=(S - 100, 2))]) for _ in range(4)])
    return np.concatenate([window, new]).astype(np.float32), W, S


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("cell_mult", [1, 2])
def test_forest_reuse_matches_oracle(precision, cell_mult):
    pts, W, S = reuse_stream()
    eps, mp = 0.25, 5
    got = run_stream(pts, W, S, eps, mp, 4, precision=precision, cell_mult=cell_mult)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    exp = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=4)
    assert_same(got[:3], exp, f"reuse/{precision}/K{cell_mult}")
    # the blob components were kept from the previous slide
    assert got[3]["reused_cores"] > 1_000
    # the bridge expired in the last slide: the two blobs it joined split
    win = O.window_of(pts, W, S, 4)
    lab, cid = got[1][-1], got[2][-1]
    core = lab == 0
    a = np.argmin(((win - (0.0, 0.0)) ** 2).sum(1) + np.where(core, 0.0, 1e9))
    b = np.argmin(((win - (10.0, 0.0)) ** 2).sum(1) + np.where(core, 0.0, 1e9))
    assert cid[a] != cid[b]


# Two grid cells per Eps: a (2K+1)^d = 5^d stencil of Eps/2 cells.  Same
# labels, ids and counts as the oracle on every case shape: 1-D, 2-D, 3-D,
# S = W, multi-chunk slides, FP32-band pairs, MinPts above the list cap.
K2_CASES = [c for c in CASES if c[0] in ("mix2d_W10k_S1k", "walk3d_W60k_S6k", "band3d_W20k_S2k", "stk1d_W8k_S2k",
                                          "big_stride_W40k_S20k", "S_eq_W_3d", "mix2d_mp40_W8k")]


@pytest.mark.parametrize("name,gen,W,S,eps,mp,slides", K2_CASES, ids=[c[0] for c in K2_CASES])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_two_cells_per_eps_match_oracle(name, gen, W, S, eps, mp, slides, precision):
    pts = gen()
    got = run_stream(pts, W, S, eps, mp, slides, precision=precision, cell_mult=2)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    exp = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, f"{name}/{precision}/K2")


# Edge shapes: one-point strides, tiny windows (down to one slot), MinPts 1
# (every point core) and 2 (empty neighbour lists), duplicates at one
# location, 1-D.
EDGE_CASES = [
    ("S1_W64_2d", lambda: wl.gaussian_mixture(64 + 40, dim=2, k=2, box=3.0, seed=41), 64, 1, 0.5, 4),
    ("mp1_3d", lambda: wl.gaussian_mixture(2_000 + 3 * 200, dim=3, k=4, box=10.0, seed=42), 2_000, 200, 0.8, 1),
    ("mp2_2d", lambda: wl.gaussian_mixture(2_000 + 3 * 200, dim=2, k=4, box=40.0, seed=43), 2_000, 200, 0.3, 2),
    ("dups_1d", lambda: np.repeat(np.linspace(0, 5, 300, dtype=np.float32)[:, None], 4, axis=0), 800, 100, 0.02, 5),
    # the smallest windows: one slot, two slots with MinPts 2, one chunk of three 1-D points
    ("W1_S1_2d", lambda: wl.gaussian_mixture(1 + 30, dim=2, k=2, box=2.0, seed=71), 1, 1, 0.5, 1),
    ("W2_S1_3d", lambda: wl.gaussian_mixture(2 + 30, dim=3, k=2, box=2.0, seed=72), 2, 1, 0.5, 2),
    ("W3_S3_1d", lambda: wl.gaussian_mixture(3 + 30, dim=1, k=2, box=2.0, seed=73), 3, 3, 0.5, 2),
]


@pytest.mark.parametrize("name,gen,W,S,eps,mp", EDGE_CASES, ids=[c[0] for c in EDGE_CASES])
@pytest.mark.parametrize("cell_mult", [1, 2])
def test_edge_shapes_match_oracle(name, gen, W, S, eps, mp, cell_mult):
    pts = gen()
    slides = (len(pts) - W) // S
    got = run_stream(pts, W, S, eps, mp, slides, cell_mult=cell_mult)
    exp = O.stream(pts, W, S, eps, mp, O.MODE_FP64, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, f"{name}/K{cell_mult}")


# Streams slid past W/S slides: every expiring chunk then arrived by a slide,
# so its (key, slot) order is the one kept from that slide and its words are
# not sorted again.  Covers one and two sort chunks per slide, S = 1 and
# S = W, both cell multipliers and both predicates.
STEADY_CASES = [
    ("mix2d_W2k_S200", lambda: wl.gaussian_mixture(2_000 + 25 * 200, dim=2, k=6, box=20.0, seed=51),
     2_000, 200, 0.5, 5, 25),
    ("walk3d_W6k_S1k", lambda: wl.random_walkers(6_000 + 14 * 1_000, n_walkers=40, seed=52), 6_000, 1_000,
     3.3e-3, 10, 14),
    ("two_chunks_W40k_S20k", lambda: wl.gaussian_mixture(40_000 + 5 * 20_000, dim=2, k=30, box=100.0, seed=53),
     40_000, 20_000, 0.4, 6, 5),
    ("S1_W16_2d", lambda: wl.gaussian_mixture(16 + 40, dim=2, k=2, box=2.0, seed=54), 16, 1, 0.5, 3, 40),
    ("S_eq_W_2d", lambda: wl.gaussian_mixture(1_500 * 5, dim=2, k=4, box=12.0, seed=55), 1_500, 1_500, 0.5, 4, 4),
    # MinPts above the list cap: the label pass scans the grid
    ("mp40_W2k_S200", lambda: wl.gaussian_mixture(2_000 + 24 * 200, dim=2, k=5, box=15.0, seed=58),
     2_000, 200, 0.8, 40, 24),
]


@pytest.mark.parametrize("name,gen,W,S,eps,mp,slides", STEADY_CASES, ids=[c[0] for c in STEADY_CASES])
@pytest.mark.parametrize("precision,cell_mult", [("fp64", 1), ("fp32", 1), ("fp64", 2)])
def test_steady_state_streams_match_oracle(name, gen, W, S, eps, mp, slides, precision, cell_mult):
    assert slides > W // S
    pts = gen()
    got = run_stream(pts, W, S, eps, mp, slides, precision=precision, cell_mult=cell_mult)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    exp = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, f"{name}/{precision}/K{cell_mult}")
    assert got[3]["error_bits"] == 0


def test_reload_after_steady_state():
    """A new first window loaded into an engine that already slid past W/S
    slides starts over: its first W/S slides sort the expired words again."""
    W, S, eps, mp = 1_200, 300, 0.5, 5
    a = wl.gaussian_mixture(W + 9 * S, dim=2, k=5, box=15.0, seed=56)
    b = wl.gaussian_mixture(W + 7 * S, dim=2, k=5, box=15.0, seed=57)
    with Engine(2, W, S, eps, mp) as eng:
        eng.load_window(a[:W])
        for k in range(9):
            eng.slide(a[W + k * S: W + (k + 1) * S])
        eng.load_window(b[:W])
        got = []
        for k in range(7):
            lab, cid = eng.slide(b[W + k * S: W + (k + 1) * S])
            got.append((eng.counts(), lab, cid))
    exp = O.stream(b, W, S, eps, mp, O.MODE_FP64, first_slide=1, n_out=7)
    assert_same(tuple(np.array(x) for x in zip(*got)), exp, "reloaded")


def duplicate_points(n, dim, seed):
    """n points on n // 3 distinct locations, each taken three times, shuffled."""
    rng = np.random.default_rng(seed)
    base = rng.uniform(-5.0, 5.0, size=(n // 3 + 1, dim)).astype(np.float32)
    pts = np.repeat(base, 3, axis=0)[:n]
    return pts[rng.permutation(n)]


# Eps beyond the data's extent (every point in one cell, all pairs tested;
# Eps^2 above 2^100 turns the FP32 filter off) and below any distance but 0
# (Eps^2 below 2^-100: the filter is off, only duplicates are neighbours).
@pytest.mark.parametrize("eps", [50.0, 1e16, 1e-31], ids=["eps_beyond_extent", "eps_1e16", "eps_1e-31"])
@pytest.mark.parametrize("precision,cell_mult", [("fp64", 1), ("fp32", 1), ("fp64", 2)])
def test_extreme_eps_match_oracle(eps, precision, cell_mult):
    W, S, mp, slides = 600, 100, 3, 8
    pts = duplicate_points(W + slides * S, 3, seed=61)
    got = run_stream(pts, W, S, eps, mp, slides, precision=precision, cell_mult=cell_mult)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    exp = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, f"eps {eps}/{precision}/K{cell_mult}")
    if eps > 1.0:
        assert np.all(got[1] == 0)  # one cluster of cores


# The count passes' block shape: a whole warp per expired or new point
# instead of a 16-lane half (one cell per Eps).
LANES_CASES = [c for c in CASES if c[0] in ("mix2d_W10k_S1k", "walk3d_W60k_S6k", "band3d_W20k_S2k", "stk1d_W8k_S2k",
                                            "big_stride_W40k_S20k", "mix3d_mp32_W12k")] + \
    [c for c in STEADY_CASES if c[0] in ("mix2d_W2k_S200", "S1_W16_2d")]


@pytest.mark.parametrize("name,gen,W,S,eps,mp,slides", LANES_CASES, ids=[c[0] for c in LANES_CASES])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_count_passes_with_whole_warp_queries(name, gen, W, S, eps, mp, slides, precision):
    pts = gen()
    got = run_stream(pts, W, S, eps, mp, slides, precision=precision, query_lanes=32)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    exp = O.stream(pts, W, S, eps, mp, mode, first_slide=1, n_out=slides)
    assert_same(got[:3], exp, f"{name}/{precision}/32 lanes")
