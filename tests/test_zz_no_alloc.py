"""rtdbs_cluster_window_noalloc: one window clustered with no device
allocation, for callers that cannot call cudaMalloc (a host process that keeps
the GPU's memory in its own pool, or a latency path that cannot take
cudaMalloc's implicit synchronisation).

Called through the C ABI and compared bit-exactly with the allocating entry
points (rtdbs_load_window + rtdbs_cluster + rtdbs_get_counts-free output) on
two calls in a row.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from rtdbstream_gb300 import Engine
from rtdbstream_gb300 import engine as E
from rtdbstream_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

MAX_POINTS = 16384


@pytest.fixture(scope="module")
def noalloc():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = E.load_library()
    fn = L.rtdbs_cluster_window_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def call_noalloc(fn, pts, eps, mp, precision):
    import torch

    d = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda()
    n = len(pts)
    lab = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    cid = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(d.data_ptr(), n, pts.shape[1], float(eps), int(mp),
            E.PREC_FP64 if precision == "fp64" else E.PREC_FP32, lab.data_ptr(), cid.data_ptr(), stream)
    assert rc == 0, f"rtdbs_cluster_window_noalloc returned {rc}"
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
]


@pytest.mark.parametrize("name,gen,eps,mp,precision", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_entry_points_twice(noalloc, name, gen, eps, mp, precision):
    pts = gen()
    exp_lab, exp_cid = call_engine(pts, eps, mp, precision)
    # an unrelated call first, so the second call of this case starts from a
    # scratch array that holds another window's data
    other = wl.gaussian_mixture(3_000, dim=3, k=5, box=10.0, seed=99)
    for k in range(2):
        lab, cid = call_noalloc(noalloc, pts, eps, mp, precision)
        assert np.array_equal(lab, exp_lab), f"{name}: labels differ on call {k + 1}"
        assert np.array_equal(cid, exp_cid), f"{name}: ids differ on call {k + 1}"
        call_noalloc(noalloc, other, 0.7, 4, "fp64")


def test_noalloc_rejects_oversized_window(noalloc):
    import torch

    n = MAX_POINTS + 1
    d = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = noalloc(d.data_ptr(), n, 2, 0.5, 4, E.PREC_FP64, out.data_ptr(), out.data_ptr(), None)
    assert rc == E.RTDBS_ERR_INVALID
