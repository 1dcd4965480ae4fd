"""The reference-compatible command line on a GPU: a tao-format stream, the
reference's arguments, the "[Time] total" line, and the last window's labels
equal to the reference-semantics (FP32) oracle."""
import subprocess

import numpy as np
import pytest

import oracle as O
from rtdbstream_gb300 import build as rbuild
from rtdbstream_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cells_per_eps,query_lanes", [(1, 16), (2, 32), (1, 32)])
def test_cli_tao_stream(tmp_path, cells_per_eps, query_lanes):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    O.build(ref=False)
    rbuild.build()
    pts = wl.gaussian_mixture(3_000, dim=3, k=6, box=15.0, seed=31)
    path = tmp_path / "tao_cli.txt"
    path.write_text("".join(f"{x!r},{y!r},{z!r}\n" for x, y, z in pts.astype(np.float64).tolist()))
    out = tmp_path / "labels.bin"
    W, S, K, R = 1_000, 250, 5, 1.0
    r = subprocess.run([rbuild.CLI, "-f", str(path), "-n", "3000", "-W", str(W), "-S", str(S), "-K", str(K),
                        "-R", str(R), "--labels", str(out), "--cells-per-eps", str(cells_per_eps),
                        "--query-lanes", str(query_lanes)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "[Time] total:" in r.stdout
    slides = (3_000 - W) // S
    got = np.fromfile(out, dtype=np.int32).reshape(W, 2)
    # the reference reads doubles and keeps floats: same float32 points
    _, elab, ecid = O.stream(pts, W, S, R, K, O.MODE_FP32, first_slide=slides, n_out=1)
    assert np.array_equal(got[:, 0], elab[0])
    keep = elab[0] != 2
    assert np.array_equal(got[keep, 1], ecid[0][keep])
