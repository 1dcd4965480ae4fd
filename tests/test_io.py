"""Dataset readers for the reference's formats (src/dbscan/util.cpp:12-254)
and the reference-compatible command line, without a GPU."""
import os
import subprocess

import numpy as np
import pytest

from rtdbstream_gb300 import build as rbuild
from rtdbstream_gb300 import engine as E


def write_formats(tmp_path, pts3):
    rng = np.random.default_rng(0)
    files = {}
    p = tmp_path / "tao_test.txt"
    p.write_text("".join(f"{x!r},{y!r},{z!r}\n" for x, y, z in pts3.astype(np.float64).tolist()))
    files["tao"] = (p, pts3, 3)
    p = tmp_path / "geolife_test.bin"
    pts3.astype(np.float64).tofile(p)
    files["geolife"] = (p, pts3, 3)
    p = tmp_path / "RBF_test.csv"
    p.write_text("x,y\n" + "".join(f"{x!r},{y!r}\n" for x, y in pts3[:, :2].astype(np.float64).tolist()))
    files["rbf"] = (p, pts3[:, :2], 2)
    p = tmp_path / "EDS_test.txt"
    ids = rng.integers(0, 9, len(pts3))
    p.write_text("id x y cid\n" + "".join(f"{i} {x!r} {y!r} {c}\n" for i, (x, y), c in
                                          zip(range(len(pts3)), pts3[:, :2].astype(np.float64).tolist(),
                                              ids.tolist())))
    files["eds"] = (p, pts3[:, :2], 2)
    p = tmp_path / "stock_test.txt"
    p.write_text("price\n" + "".join(f"{x!r}\n" for x in pts3[:, 0].astype(np.float64).tolist()))
    files["stock"] = (p, pts3[:, :1], 1)
    return files


@pytest.mark.parametrize("fmt", ["tao", "geolife", "rbf", "eds", "stock"])
def test_readers_match_numpy(tmp_path, fmt):
    pts3 = np.random.default_rng(1).normal(10.0, 3.0, (257, 3)).astype(np.float32)
    path, exp, dim = write_formats(tmp_path, pts3)[fmt]
    for f in ("auto", fmt):  # the file name selects the format, like the reference
        got, lo, hi = E.read_points(str(path), 1000, f)
        assert got.shape == (257, dim)
        assert np.array_equal(got, exp)
        assert np.array_equal(lo, exp.min(axis=0)) and np.array_equal(hi, exp.max(axis=0))
    got, _, _ = E.read_points(str(path), 100, fmt)  # -n limits the points read
    assert np.array_equal(got, exp[:100])


def test_reader_errors(tmp_path):
    with pytest.raises(E.RtdbsError):
        E.read_points(str(tmp_path / "missing_tao.txt"), 10)
    p = tmp_path / "unknown.txt"
    p.write_text("1,2,3\n")
    with pytest.raises(E.RtdbsError):
        E.read_points(str(p), 10)  # no format in the name


def cli():
    rbuild.build()
    return rbuild.CLI


def test_cli_usage_and_bad_dataset(tmp_path):
    r = subprocess.run([cli()], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stderr
    r = subprocess.run([cli(), "-f", str(tmp_path / "tao_missing.txt"), "-n", "100", "-W", "10", "-S", "5",
                        "-K", "3", "-R", "0.5"], capture_output=True, text=True)
    assert r.returncode == 2 and "cannot be read" in r.stderr
