"""Batched pools: many uneven streams slid together, one launch per kernel
phase.  Every stream's result must be bit-identical to the same stream run
alone on the single-stream engine (and to the CPU oracle)."""
import numpy as np
import pytest

import oracle as O
from rtdbstream_gb300 import Engine, Pool, RtdbsError, make_params, stream_bytes
from rtdbstream_gb300 import engine as E
from rtdbstream_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    O.build(ref=False)
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


# (dim, W, S, eps, min_pts, precision, generator)
STREAMS = [
    (2, 4_000, 400, 0.5, 5, "fp64", lambda n, s: wl.gaussian_mixture(n, dim=2, k=8, box=30.0, seed=s)),
    (3, 12_000, 1_200, 3.3e-3, 10, "fp64", lambda n, s: wl.random_walkers(n, n_walkers=24, seed=s)),
    (2, 1_000, 100, 0.4, 4, "fp32", lambda n, s: wl.gaussian_mixture(n, dim=2, k=4, box=15.0, seed=s)),
    (1, 6_000, 2_000, 0.01, 4, "fp64",
     lambda n, s: wl.gaussian_mixture(n, dim=1, k=6, box=10.0, sigma=0.3, seed=s)),
    (3, 40_000, 20_000, 0.6, 6, "fp64", lambda n, s: wl.gaussian_mixture(n, dim=3, k=30, box=40.0, seed=s)),
    (3, 3_000, 3_000, 1.0, 5, "fp32", lambda n, s: wl.gaussian_mixture(n, dim=3, k=6, box=15.0, seed=s)),
    (3, 8_000, 800, 1e-3, 2, "fp64",
     lambda n, s: wl.offset_band_points(n, 1e-3, partner_frac=0.3, seed=s)),
    (2, 20_000, 1_000, 0.35, 8, "fp64", lambda n, s: wl.gaussian_mixture(n, dim=2, k=20, box=60.0, seed=s)),
]
ROUNDS = 3


def stream_data():
    return [gen(W + ROUNDS * S, 100 + i) for i, (dim, W, S, eps, mp, prec, gen) in enumerate(STREAMS)]


def solo(pts, dim, W, S, eps, mp, prec, rounds):
    out = []
    with Engine(dim, W, S, eps, mp, precision=prec) as eng:
        eng.load_window(pts[:W])
        for k in range(rounds):
            lab, cid = eng.slide(pts[W + k * S: W + (k + 1) * S])
            out.append((lab, cid, eng.counts()))
    return out


def packed(data, ids, k):
    import torch

    parts = []
    for i in ids:
        dim, W, S = STREAMS[i][:3]
        parts.append(data[i][W + k * S: W + (k + 1) * S].reshape(-1))
    return torch.from_numpy(np.concatenate(parts)).cuda()


@pytest.mark.parametrize("use_graph", [True, False])
def test_pool_matches_solo_engines(use_graph):
    data = stream_data()
    with Pool(use_graph=use_graph) as pool:
        sids = []
        for i, (dim, W, S, eps, mp, prec, _) in enumerate(STREAMS):
            sid = pool.add_stream(make_params(dim, W, S, eps, mp, precision=prec))
            pool.load_window(sid, data[i][:W])
            sids.append(sid)
        got = [[] for _ in STREAMS]
        for k in range(ROUNDS):
            pool.slide(sids, packed(data, range(len(STREAMS)), k))
            pool.sync()
            for i, sid in enumerate(sids):
                lab, cid = pool.outputs(sid)
                got[i].append((lab, cid, pool.counts(sid)))
        st = pool.stats()
        if use_graph:
            assert st["graph_replays"] == ROUNDS - 1
    for i, (dim, W, S, eps, mp, prec, _) in enumerate(STREAMS):
        ref = solo(data[i], dim, W, S, eps, mp, prec, ROUNDS)
        for k in range(ROUNDS):
            for a, b, what in zip(got[i][k], ref[k], ("label", "cid", "count")):
                assert np.array_equal(a, b), f"stream {i} round {k}: {what} differs"


def test_pool_subset_rounds_and_oracle():
    """Rounds over changing subsets: a stream that sits out keeps its window."""
    data = stream_data()
    sel = [0, 1, 2, 6]
    with Pool() as pool:
        sids = {}
        for i in sel:
            dim, W, S, eps, mp, prec, _ = STREAMS[i]
            sids[i] = pool.add_stream(make_params(dim, W, S, eps, mp, precision=prec))
            pool.load_window(sids[i], data[i][:W])
        schedule = [[0, 1, 2, 6], [1, 6], [0, 2], [0, 1, 2, 6]]
        done = {i: 0 for i in sel}
        for members in schedule:
            pool.slide([sids[i] for i in members], packed_at(data, members, done))
            pool.sync()
            for i in members:
                done[i] += 1
            for i in members:
                dim, W, S, eps, mp, prec, _ = STREAMS[i]
                mode = O.MODE_FP64 if prec == "fp64" else O.MODE_FP32
                exp = O.stream(data[i], W, S, eps, mp, mode, first_slide=done[i], n_out=1)
                lab, cid = pool.outputs(sids[i])
                assert np.array_equal(lab, exp[1][0]) and np.array_equal(cid, exp[2][0])
                assert np.array_equal(pool.counts(sids[i]), exp[0][0])


def packed_at(data, members, done):
    import torch

    parts = []
    for i in members:
        dim, W, S = STREAMS[i][:3]
        k = done[i]
        parts.append(data[i][W + k * S: W + (k + 1) * S].reshape(-1))
    return torch.from_numpy(np.concatenate(parts)).cuda()


def test_pool_admission_by_budget():
    p = make_params(3, 50_000, 5_000, 1e-3, 5)
    one = stream_bytes(p)
    with Pool(hbm_budget_bytes=2 * one + one // 2) as pool:
        a = pool.add_stream(p)
        b = pool.add_stream(p)
        with pytest.raises(RtdbsError) as ei:
            pool.add_stream(p)
        assert ei.value.status == E.RTDBS_ERR_BUDGET
        pool.remove_stream(a)
        c = pool.add_stream(p)  # the freed memory admits a new stream
        assert pool.stats()["streams"] == 2 and pool.stats()["bytes_in_use"] == 2 * one
        assert c == a and b != a


def test_pool_rejects_unloaded_and_duplicate_streams():
    import torch

    with Pool() as pool:
        sid = pool.add_stream(make_params(2, 1_000, 100, 0.5, 4))
        d = torch.zeros(200 * 2, dtype=torch.float32, device="cuda")
        with pytest.raises(RtdbsError) as ei:
            pool.slide([sid], d)
        assert ei.value.status == E.RTDBS_ERR_STATE
        pool.load_window(sid, np.zeros((1_000, 2), np.float32))
        with pytest.raises(RtdbsError) as ei:
            pool.slide([sid, sid], d)
        assert ei.value.status == E.RTDBS_ERR_INVALID


def test_pool_mixes_cell_multipliers():
    """Streams with one and two cells per Eps (separate launch groups) and
    with 16 or 32 lanes per count query (one group, a block shape per stream)
    in one pool equal the same streams alone and the oracle."""
    specs = [(2, 4_000, 400, 0.5, 5, (1, 0)), (2, 4_000, 400, 0.5, 5, (2, 0)), (3, 6_000, 600, 0.8, 6, (2, 0)),
             (3, 6_000, 600, 0.8, 6, (1, 0)), (2, 4_000, 400, 0.5, 5, (1, 32)), (3, 6_000, 600, 0.8, 6, (1, 32))]
    data = [wl.gaussian_mixture(W + ROUNDS * S, dim=dim, k=6, box=20.0, seed=300 + i)
            for i, (dim, W, S, eps, mp, km) in enumerate(specs)]

    def shape(km):  # (cells per Eps, lanes per count query)
        return {"cell_mult": km[0], "query_lanes": km[1]}

    import torch

    with Pool() as pool:
        ids = []
        for (dim, W, S, eps, mp, km), d in zip(specs, data):
            sid = pool.add_stream(make_params(dim, W, S, eps, mp, **shape(km)))
            pool.load_window(sid, d[:W])
            ids.append(sid)
        for k in range(ROUNDS):
            buf = torch.from_numpy(np.concatenate([d[W + k * S: W + (k + 1) * S].reshape(-1)
                                                   for (dim, W, S, eps, mp, km), d in zip(specs, data)])).cuda()
            pool.slide(ids, buf)
        for sid, (dim, W, S, eps, mp, km), d in zip(ids, specs, data):
            lab, cid = pool.outputs(sid)
            with Engine(dim, W, S, eps, mp, **shape(km)) as eng:
                eng.load_window(d[:W])
                for k in range(ROUNDS):
                    elab, ecid = eng.slide(d[W + k * S: W + (k + 1) * S])
            assert np.array_equal(lab, elab) and np.array_equal(cid, ecid)
            win = O.window_of(d, W, S, ROUNDS)
            _, olab, ocid, _ = O.window_grid(win, eps, mp, O.MODE_FP64)
            assert np.array_equal(lab, olab) and np.array_equal(cid, ocid)


def test_pool_steady_state_rounds():
    """Pool streams slid past W/S rounds (expired chunks in their kept order,
    not sorted again), one of them sitting out every third round, against the
    oracle after each round."""
    import torch

    specs = [(2, 1_000, 100, 0.5, 5, 1), (3, 2_400, 800, 0.8, 6, 1), (2, 1_200, 150, 0.5, 4, 2)]
    rounds = 16
    data = [wl.gaussian_mixture(W + rounds * S, dim=dim, k=5, box=15.0, seed=310 + i)
            for i, (dim, W, S, eps, mp, km) in enumerate(specs)]
    done = [0] * len(specs)
    with Pool() as pool:
        ids = []
        for (dim, W, S, eps, mp, km), d in zip(specs, data):
            sid = pool.add_stream(make_params(dim, W, S, eps, mp, cell_mult=km))
            pool.load_window(sid, d[:W])
            ids.append(sid)
        for r in range(rounds):
            members = [i for i in range(len(specs)) if not (i == 1 and r % 3 == 2)]
            buf = torch.from_numpy(np.concatenate([data[i][specs[i][1] + done[i] * specs[i][2]:
                                                           specs[i][1] + (done[i] + 1) * specs[i][2]].reshape(-1)
                                                   for i in members])).cuda()
            pool.slide([ids[i] for i in members], buf)
            pool.sync()
            for i in members:
                done[i] += 1
                dim, W, S, eps, mp, km = specs[i]
                win = O.window_of(data[i], W, S, done[i])
                enn, elab, ecid, _ = O.window_grid(win, eps, mp, O.MODE_FP64)
                lab, cid = pool.outputs(ids[i])
                assert np.array_equal(lab, elab) and np.array_equal(cid, ecid), f"stream {i} round {r}"
                assert np.array_equal(pool.counts(ids[i]), enn), f"stream {i} round {r}: counts"
    assert min(done) > max(W // S for dim, W, S, *_ in specs)


def test_pool_mixes_list_and_grid_label_streams():
    """Streams with MinPts above the neighbour-list cap (label pass scans the
    grid, no forest reuse) next to list streams in one pool, over enough
    rounds to pass W/S: each equals the oracle after every round."""
    import torch

    specs = [(2, 1_500, 150, 0.8, 40, "fp64"), (2, 1_500, 150, 0.5, 5, "fp64"), (3, 2_000, 250, 1.2, 36, "fp32"),
             (3, 2_000, 250, 0.8, 6, "fp32")]
    rounds = 12
    data = [wl.gaussian_mixture(W + rounds * S, dim=dim, k=4, box=12.0, seed=330 + i)
            for i, (dim, W, S, eps, mp, prec) in enumerate(specs)]
    with Pool() as pool:
        ids = []
        for (dim, W, S, eps, mp, prec), d in zip(specs, data):
            sid = pool.add_stream(make_params(dim, W, S, eps, mp, precision=prec))
            pool.load_window(sid, d[:W])
            ids.append(sid)
        for r in range(rounds):
            buf = torch.from_numpy(np.concatenate([d[W + r * S: W + (r + 1) * S].reshape(-1)
                                                   for (dim, W, S, eps, mp, prec), d in zip(specs, data)])).cuda()
            pool.slide(ids, buf)
            pool.sync()
            for sid, (dim, W, S, eps, mp, prec), d in zip(ids, specs, data):
                mode = O.MODE_FP64 if prec == "fp64" else O.MODE_FP32
                enn, elab, ecid, _ = O.window_grid(O.window_of(d, W, S, r + 1), eps, mp, mode)
                lab, cid = pool.outputs(sid)
                assert np.array_equal(pool.counts(sid), enn), f"MinPts {mp} round {r}: counts"
                assert np.array_equal(lab, elab) and np.array_equal(cid, ecid), f"MinPts {mp} round {r}"
