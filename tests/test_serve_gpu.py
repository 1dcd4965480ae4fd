"""Continuous-batching server: results equal the stream run alone (CPU oracle
replay of exactly the slides each stream received), and streams beyond the
HBM budget are admitted as earlier streams finish and free their memory."""
import numpy as np
import pytest

import oracle as O
from rtdbstream_gb300 import make_params, stream_bytes
from rtdbstream_gb300 import workloads as wl
from rtdbstream_gb300.serve import ServedStream, SlideServer, poisson_arrivals

pytestmark = pytest.mark.gpu

K = 3  # distinct slides of data per stream (reused cyclically)


@pytest.fixture(scope="module")
def torch_stream():
    O.build(ref=False)
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    s = torch.cuda.Stream()
    prev = torch.cuda.current_stream()
    torch.cuda.set_stream(s)
    yield s
    torch.cuda.set_stream(prev)


def make_streams(n, seed):
    import torch

    specs = wl.mixed_streams(n, seed=seed, w_lo=1_000, w_hi=20_000)
    out = []
    for sp in specs:
        pts = wl.mix_points(sp, sp.window + K * sp.stride)
        data = torch.from_numpy(np.ascontiguousarray(pts[sp.window:]).reshape(K, sp.stride * sp.dim)).cuda()
        out.append((sp, pts, ServedStream(sp, pts[:sp.window], data)))
    return out


def replay(sp, pts, done):
    """The window a stream holds after `done` slides of cyclically reused data."""
    seq = [pts[:sp.window]] + [pts[sp.window + (k % K) * sp.stride: sp.window + (k % K + 1) * sp.stride]
                               for k in range(done)]
    return O.window_of(np.concatenate(seq), sp.window, sp.stride, done)


def test_server_results_match_streams_alone(torch_stream):
    streams = make_streams(16, seed=11)
    srv = SlideServer(stream=torch_stream.cuda_stream)
    for _, _, st in streams:
        srv.add(st)
    t, tgt = poisson_arrivals(rate=400.0, duration=0.5, n_streams=len(streams), seed=5)
    res = srv.run(t, tgt)
    assert res["requests"] == len(t)
    assert res["mean_round_size"] >= 1.0
    for sp, pts, st in streams:
        if st.done == 0:
            continue
        win = replay(sp, pts, st.done)
        _, elab, ecid, _ = O.window_grid(win, sp.eps, sp.min_pts, O.MODE_FP64)
        lab, cid = srv.pool.outputs(st.sid)
        assert np.array_equal(lab, elab) and np.array_equal(cid, ecid)
    srv.close()


def test_server_admits_as_memory_frees(torch_stream):
    streams = make_streams(12, seed=12)
    costs = [stream_bytes(make_params(sp.dim, sp.window, sp.stride, sp.eps, sp.min_pts)) for sp, _, _ in streams]
    budget = sum(sorted(costs)[-4:]) + 1        # any 4 streams fit, not all 12
    srv = SlideServer(hbm_budget_bytes=budget, stream=torch_stream.cuda_stream)
    t, tgt = poisson_arrivals(rate=300.0, duration=0.4, n_streams=len(streams), seed=6)
    per = np.bincount(tgt, minlength=len(streams))
    for (sp, pts, st), n_req in zip(streams, per):
        st.requests_total = int(n_req) if n_req else 1
        srv.add(st)
    assert len(srv.waiting) > 0                 # the budget holds some streams back
    # streams without requests would never leave: give each one request
    extra_t = [t.max() + 0.01 * (i + 1) for i, n_req in enumerate(per) if n_req == 0]
    extra_i = [i for i, n_req in enumerate(per) if n_req == 0]
    t2 = np.concatenate([t, np.asarray(extra_t)]) if extra_t else t
    tgt2 = np.concatenate([tgt, np.asarray(extra_i, dtype=tgt.dtype)]) if extra_t else tgt
    order = np.argsort(t2, kind="stable")
    res = srv.run(t2[order], tgt2[order])
    assert res["requests"] == len(t2)
    assert not srv.waiting and all(st.sid is None for _, _, st in streams)
    assert srv.pool.stats()["streams"] == 0
    srv.close()


def test_budget_bound_results_match_streams_alone(torch_stream):
    """The mix is bigger than the budget: streams wait, are admitted as
    others finish, and every stream's final window is still exact."""
    streams = make_streams(20, seed=13)
    costs = [stream_bytes(make_params(sp.dim, sp.window, sp.stride, sp.eps, sp.min_pts)) for sp, _, _ in streams]
    budget = sum(sorted(costs)[-5:]) + 1        # any 5 streams fit, not all 20
    srv = SlideServer(hbm_budget_bytes=budget, stream=torch_stream.cuda_stream, depth=2)
    t, tgt = poisson_arrivals(rate=600.0, duration=0.4, n_streams=len(streams), seed=7)
    # every stream also gets 2..4 requests appended after the Poisson ones
    rng = np.random.default_rng(8)
    extra = np.repeat(np.arange(len(streams)), rng.integers(2, 5, len(streams)))
    t2 = np.concatenate([t, t.max() + 0.001 * np.arange(1, len(extra) + 1)])
    tgt2 = np.concatenate([tgt, extra.astype(tgt.dtype)])
    per = np.bincount(tgt2, minlength=len(streams))
    for (sp, pts, st), n_req in zip(streams, per):
        st.requests_total = int(n_req)
        srv.add(st)
    assert len(srv.waiting) > 0
    # every stream's final result, read just before it leaves the pool
    finals = {}
    orig_retire = srv._retire

    def retire_and_keep(i):
        finals[i] = srv.pool.outputs(srv.streams[i].sid)
        orig_retire(i)

    srv._retire = retire_and_keep
    res = srv.run(t2, tgt2)
    assert res["requests"] == len(t2)
    assert res["admission_wait_ms_p50"] is not None
    assert not srv.waiting and srv.pool.stats()["streams"] == 0
    for i, (sp, pts, st) in enumerate(streams):
        assert st.done == per[i]
        win = replay(sp, pts, st.done)
        _, elab, ecid, _ = O.window_grid(win, sp.eps, sp.min_pts, O.MODE_FP64)
        lab, cid = finals[i]
        assert np.array_equal(lab, elab) and np.array_equal(cid, ecid), f"stream {i}"
    srv.close()


def test_budget_refusals(torch_stream):
    """A stream larger than the whole budget is refused when added; requests
    that only waiting streams could serve, with nothing left to free memory,
    end the run with RTDBS_ERR_BUDGET instead of waiting forever."""
    from rtdbstream_gb300 import RtdbsError
    from rtdbstream_gb300.engine import RTDBS_ERR_BUDGET

    streams = make_streams(3, seed=14)
    costs = [stream_bytes(make_params(sp.dim, sp.window, sp.stride, sp.eps, sp.min_pts)) for sp, _, _ in streams]
    srv = SlideServer(hbm_budget_bytes=min(costs) - 1, stream=torch_stream.cuda_stream)
    with pytest.raises(RtdbsError) as e:
        srv.add(streams[int(np.argmin(costs))][2])
    assert e.value.status == RTDBS_ERR_BUDGET
    srv.close()
    # budget for one stream: the first is admitted (no request limit and no
    # requests), the second waits and has requests
    order = np.argsort(costs)[::-1]
    a, b = streams[order[0]][2], streams[order[1]][2]
    srv = SlideServer(hbm_budget_bytes=costs[order[0]] + 1, stream=torch_stream.cuda_stream)
    srv.add(a)
    srv.add(b)
    assert a.sid is not None and b.sid is None
    with pytest.raises(RtdbsError) as e:
        srv.run(np.array([0.0, 0.001]), np.array([1, 1]))
    assert e.value.status == RTDBS_ERR_BUDGET
    srv.close()
