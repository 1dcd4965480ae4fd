"""rtdbs_cluster_window_noalloc: one window clustered with no device
allocation, for callers that cannot call cudaMalloc (a host process that keeps
the GPU's memory in its own pool, or a latency path that cannot take
cudaMalloc's implicit synchronisation).

Called through the C ABI and compared bit-exactly with the allocating entry
points (rtdbs_load_window + rtdbs_cluster) and with the CPU oracle on two
calls in a row, with another window clustered in between.  Also checks that a
warm call leaves the device's free memory unchanged, and that a call works as
the first kernel launch of a fresh process.  The variant without waits
(rtdbs_cluster_window_noalloc_async) is compared with the oracle with a box
around and a box inside the data, and replayed from a captured CUDA graph on
new points.  This file is collected last on purpose.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
from rtdbstream_gb300 import Engine
from rtdbstream_gb300 import engine as E
from rtdbstream_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

MAX_POINTS = 16384
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def noalloc():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    O.build(ref=False)
    L = E.load_library()
    fn = L.rtdbs_cluster_window_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def device_buffers(pts):
    import torch

    d = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda()
    n = len(pts)
    lab = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    cid = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    return d, lab, cid


def call_noalloc(fn, pts, eps, mp, precision, bufs=None):
    import torch

    d, lab, cid = bufs or device_buffers(pts)
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(d.data_ptr(), len(pts), pts.shape[1], float(eps), int(mp),
            E.PREC_FP64 if precision == "fp64" else E.PREC_FP32, lab.data_ptr(), cid.data_ptr(), stream)
    assert rc == 0, f"rtdbs_cluster_window_noalloc returned {rc}: {E.load_library().rtdbs_last_error()}"
    return lab.cpu().numpy(), cid.cpu().numpy()


def call_engine(pts, eps, mp, precision):
    n = len(pts)
    with Engine(pts.shape[1], n, n, eps, mp, precision=precision) as eng:
        eng.load_window(np.ascontiguousarray(pts, np.float32))
        return eng.cluster()


CASES = [
    ("mix2d", lambda: wl.gaussian_mixture(6_000, dim=2, k=8, box=25.0, seed=41), 0.5, 5, "fp64"),
    ("walk3d_max", lambda: wl.random_walkers(MAX_POINTS, n_walkers=40, seed=42), 3.3e-3, 10, "fp64"),
    ("band3d_fp32", lambda: wl.offset_band_points(5_000, 1e-3, partner_frac=0.3, seed=43), 1e-3, 2, "fp32"),
    ("stk1d", lambda: wl.gaussian_mixture(4_000, dim=1, k=6, box=10.0, sigma=0.3, seed=44), 0.01, 4, "fp64"),
    ("mix3d_mp40", lambda: wl.gaussian_mixture(8_000, dim=3, k=6, box=12.0, seed=45), 0.9, 40, "fp64"),
]


@pytest.mark.parametrize("name,gen,eps,mp,precision", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_engine_and_oracle_twice(noalloc, name, gen, eps, mp, precision):
    pts = gen()
    exp_lab, exp_cid = call_engine(pts, eps, mp, precision)
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    _, o_lab, o_cid, _ = O.window_grid(pts, eps, mp, mode)
    assert np.array_equal(exp_lab, o_lab) and np.array_equal(exp_cid, o_cid), f"{name}: engine vs oracle"
    # an unrelated call between the two, so the second call of this case
    # starts from a scratch array that holds another window's data
    other = wl.gaussian_mixture(3_000, dim=3, k=5, box=10.0, seed=99)
    for k in range(2):
        lab, cid = call_noalloc(noalloc, pts, eps, mp, precision)
        assert np.array_equal(lab, o_lab), f"{name}: labels differ from the oracle on call {k + 1}"
        assert np.array_equal(cid, o_cid), f"{name}: ids differ from the oracle on call {k + 1}"
        assert np.array_equal(lab, exp_lab) and np.array_equal(cid, exp_cid), f"{name}: engine, call {k + 1}"
        call_noalloc(noalloc, other, 0.7, 4, "fp64")


def test_noalloc_allocates_no_device_memory(noalloc):
    import torch

    pts = wl.gaussian_mixture(MAX_POINTS, dim=3, k=10, box=20.0, seed=46)
    bufs = device_buffers(pts)
    call_noalloc(noalloc, pts, 0.8, 6, "fp64", bufs)  # warm: set-up done
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call_noalloc(noalloc, pts, 0.8, 6, "fp64", bufs)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"


def test_noalloc_first_kernel_launch_of_a_fresh_process(noalloc):
    """The set-up on the first call (the device address of the static
    array) works when the library has launched nothing else in the process."""
    code = r'''
import ctypes, sys
import numpy as np
sys.path.insert(0, ROOT_DIR)
from rtdbstream_gb300 import engine as E
from rtdbstream_gb300 import workloads as wl
import oracle as O
import torch  # device buffers only: the call below is the library's first launch
L = E.load_library()
fn = L.rtdbs_cluster_window_noalloc
fn.restype = ctypes.c_int
fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
               ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
pts = wl.gaussian_mixture(5_000, dim=2, k=6, box=25.0, seed=47)
n = len(pts)
d = torch.from_numpy(pts).cuda()
lab = torch.empty(n, dtype=torch.int32, device="cuda")
cid = torch.empty(n, dtype=torch.int32, device="cuda")
rc = fn(d.data_ptr(), n, 2, 0.5, 5, E.PREC_FP64, lab.data_ptr(), cid.data_ptr(), None)
assert rc == 0, (rc, L.rtdbs_last_error())
_, elab, ecid, _ = O.window_grid(pts, 0.5, 5, O.MODE_FP64)
assert np.array_equal(lab.cpu().numpy(), elab) and np.array_equal(cid.cpu().numpy(), ecid)
print("fresh-process call ok")
'''.replace("ROOT_DIR", repr(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh-process call ok" in r.stdout


def test_noalloc_rejects_oversized_window(noalloc):
    import torch

    n = MAX_POINTS + 1
    d = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = noalloc(d.data_ptr(), n, 2, 0.5, 4, E.PREC_FP64, out.data_ptr(), out.data_ptr(), None)
    assert rc == E.RTDBS_ERR_INVALID
    assert b"RTDBS_NOALLOC_MAX_POINTS" in E.load_library().rtdbs_last_error()


# ---------------------------------------------------------------- no waits
@pytest.fixture(scope="module")
def noalloc_async(noalloc):
    fn = E.load_library().rtdbs_cluster_window_noalloc_async
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    return fn


def call_async(fn, bufs, dim, eps, mp, precision, lo, hi, status, stream):
    d, lab, cid = bufs
    blo = (ctypes.c_float * 3)(*[float(x) for x in lo])
    bhi = (ctypes.c_float * 3)(*[float(x) for x in hi])
    return fn(d.data_ptr(), d.shape[0], dim, float(eps), int(mp),
              E.PREC_FP64 if precision == "fp64" else E.PREC_FP32, blo, bhi, lab.data_ptr(), cid.data_ptr(),
              status.data_ptr(), stream)


@pytest.mark.parametrize("shrink", [0.0, 0.3], ids=["data_box", "box_inside_data"])
@pytest.mark.parametrize("name,gen,eps,mp,precision", CASES[:3], ids=[c[0] for c in CASES[:3]])
def test_noalloc_async_matches_oracle(noalloc_async, name, gen, eps, mp, precision, shrink):
    """The caller's box sets the grid; with a box inside the data (points
    beyond it fall into the edge cells) the result is still exact."""
    import torch

    pts = gen()
    mode = O.MODE_FP64 if precision == "fp64" else O.MODE_FP32
    _, o_lab, o_cid, _ = O.window_grid(pts, eps, mp, mode)
    lo, hi = pts.min(axis=0).astype(np.float64), pts.max(axis=0).astype(np.float64)
    lo, hi = lo + shrink * (hi - lo), hi - shrink * (hi - lo)
    bufs = device_buffers(pts)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    rc = call_async(noalloc_async, bufs, pts.shape[1], eps, mp, precision, lo, hi, status,
                    torch.cuda.current_stream().cuda_stream)
    assert rc == 0, E.load_library().rtdbs_last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert np.array_equal(bufs[1].cpu().numpy(), o_lab), f"{name}: labels differ from the oracle"
    assert np.array_equal(bufs[2].cpu().numpy(), o_cid), f"{name}: ids differ from the oracle"


def test_noalloc_async_captured_in_a_cuda_graph(noalloc_async):
    """Captured once, replayed on new points written into the same input
    buffer: every replay equals the oracle on the points it saw."""
    import torch

    n, eps, mp = 6_000, 0.5, 5
    sets = [wl.gaussian_mixture(n, dim=2, k=8, box=25.0, seed=s) for s in (51, 52, 53)]
    lo, hi = np.zeros(3), np.full(3, 25.0)
    bufs = device_buffers(sets[0])
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):  # first call outside the capture (device set-up)
        assert call_async(noalloc_async, bufs, 2, eps, mp, "fp64", lo, hi, status, side.cuda_stream) == 0
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = call_async(noalloc_async, bufs, 2, eps, mp, "fp64", lo, hi, status,
                        torch.cuda.current_stream().cuda_stream)
    assert rc == 0, E.load_library().rtdbs_last_error()
    for pts in sets[1:] + sets[:1]:
        bufs[0].copy_(torch.from_numpy(pts))
        status.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        _, o_lab, o_cid, _ = O.window_grid(pts, eps, mp, O.MODE_FP64)
        assert int(status.item()) == 0
        assert np.array_equal(bufs[1].cpu().numpy(), o_lab) and np.array_equal(bufs[2].cpu().numpy(), o_cid)


def test_noalloc_tiny_windows(noalloc, noalloc_async):
    """One point (a core with MinPts 1, noise with 2) and an empty window."""
    import torch

    pts = np.array([[0.25, -1.5]], np.float32)
    for mp, lab in ((1, 0), (2, 2)):
        got_lab, got_cid = call_noalloc(noalloc, pts, 0.5, mp, "fp64")
        assert got_lab.tolist() == [lab] and got_cid.tolist() == [0]
        bufs = device_buffers(pts)
        status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        assert call_async(noalloc_async, bufs, 2, 0.5, mp, "fp64", pts[0], pts[0], status, None) == 0
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        assert bufs[1].cpu().tolist() == [lab] and bufs[2].cpu().tolist() == [0]
    empty = torch.empty((0, 2), dtype=torch.float32, device="cuda")
    out = torch.empty(1, dtype=torch.int32, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    assert call_async(noalloc_async, (empty, out, out), 2, 0.5, 2, "fp64", [0, 0], [1, 1], status, None) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0


def test_noalloc_async_rejects_bad_box_before_queueing(noalloc_async):
    import torch

    pts = wl.gaussian_mixture(1_000, dim=2, k=3, box=10.0, seed=54)
    bufs = device_buffers(pts)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    rc = call_async(noalloc_async, bufs, 2, 0.5, 4, "fp64", [5.0, 0.0, 0.0], [1.0, 10.0, 0.0], status, None)
    assert rc == E.RTDBS_ERR_INVALID
    torch.cuda.synchronize()
    assert int(status.item()) == -1  # nothing was queued
    assert np.all(bufs[1].cpu().numpy() == -7)
