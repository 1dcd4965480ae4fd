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
