"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, and
exports every function include/rtdbs.h declares; argument validation and
status reporting work without touching a device."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

from rtdbstream_gb300 import build as rbuild
from rtdbstream_gb300 import engine as E


def header_functions():
    text = open(os.path.join(ROOT, "include", "rtdbs.h")).read()
    return re.findall(r"RTDBS_API\s+[\w\s\*]+?\b(rtdbs_\w+)\s*\(", text)


@pytest.fixture(scope="module")
def lib():
    return E.load_library()


def test_header_declares_api():
    names = header_functions()
    assert "rtdbs_create" in names and "rtdbs_slide" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name
    assert set(header_functions()) == set(E.EXPORTED_SYMBOLS)


def test_library_is_sm103a_build():
    rbuild.build()
    assert os.path.exists(rbuild.LIB)
    assert "arch=compute_103a,code=sm_103a" in rbuild.ARCH


def test_abi_version_and_status_strings(lib):
    assert lib.rtdbs_abi_version() == 2
    assert lib.rtdbs_status_string(0) == b"ok"
    assert lib.rtdbs_status_string(-5) == b"device-side bound hit"


def test_params_init_defaults(lib):
    p = E.Params()
    assert lib.rtdbs_params_init(ctypes.byref(p)) == 0
    assert p.dim == 3 and p.precision == E.PREC_FP64 and p.has_bbox == 0


@pytest.mark.parametrize("field,value", [("dim", 4), ("dim", 0), ("stride", 7), ("eps", 0.0),
                                         ("eps", float("nan")), ("precision", 9), ("stride", 0),
                                         ("cell_mult", 3), ("cell_mult", -1), ("work_grab", 65),
                                         ("work_grab", -2), ("query_lanes", 8), ("query_lanes", 64),
                                         ("query_lanes", -16), ("two_cells_16_lanes", None)])
def test_invalid_params_rejected_before_device(lib, field, value):
    p = E.Params()
    lib.rtdbs_params_init(ctypes.byref(p))
    p.dim, p.window, p.stride, p.min_pts, p.eps = 2, 100, 10, 4, 0.5
    if field == "two_cells_16_lanes":  # the two-cells-per-Eps stencil needs the whole warp
        p.cell_mult, p.query_lanes = 2, 16
    else:
        setattr(p, field, value)
    h = ctypes.c_void_p()
    rc = lib.rtdbs_create(ctypes.byref(p), None, ctypes.byref(h))
    assert rc == E.RTDBS_ERR_INVALID
    assert lib.rtdbs_last_error() != b""
    assert not h.value


def test_null_arguments(lib):
    assert lib.rtdbs_create(None, None, None) == E.RTDBS_ERR_INVALID
    assert lib.rtdbs_slide(None, None, None, None) == E.RTDBS_ERR_INVALID
    assert lib.rtdbs_destroy(None) == 0


def test_create_without_device_fails_cleanly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = E.Params()
    lib.rtdbs_params_init(ctypes.byref(p))
    p.dim, p.window, p.stride, p.min_pts, p.eps = 2, 100, 10, 4, 0.5
    h = ctypes.c_void_p()
    assert lib.rtdbs_create(ctypes.byref(p), None, ctypes.byref(h)) == E.RTDBS_ERR_NO_DEVICE


def test_engine_raises_without_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(E.RtdbsError):
        E.Engine(2, 100, 10, 0.5, 4)


def test_stream_bytes_without_device():
    small = E.make_params(2, 1_000, 100, 0.5, 4)
    big = E.make_params(3, 1_000_000, 10_000, 3.3e-3, 10)
    a, b = E.stream_bytes(small), E.stream_bytes(big)
    assert 0 < a < b
    # dominated by the window-sized buffers: ~212 bytes per slot at W = 1M,
    # of which 40 are the neighbour lists of non-core points (MinPts 10)
    assert 180 * 1_000_000 < b < 260 * 1_000_000
    # MinPts above the longest list kept: no list buffers
    no_lists = E.stream_bytes(E.make_params(3, 1_000_000, 10_000, 3.3e-3, 40))
    assert 120 * 1_000_000 < no_lists <= b - 40 * 1_000_000


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors have the C structs' sizes and field offsets (a C
    compiler reads include/rtdbs.h)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"rtdbs_params": E.Params, "rtdbs_stats": E.Stats, "rtdbs_phase_times": E.PhaseTimes,
               "rtdbs_pool_params": E.PoolParams, "rtdbs_pool_stats": E.PoolStats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "rtdbs.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'    printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
