import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def golden_files(kind: str):
    """kind: 'window' or 'stream'."""
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))):
        is_stream = os.path.basename(f).startswith("stream_")
        if (kind == "stream") == is_stream:
            out.append(f)
    return out


def load_golden(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build(ref=True)
    return oracle


def core_partition_equal(lab_a, cid_a, lab_b, cid_b):
    """True when the core points carry identical canonical ids (the minimum
    core slot of each component) in both results."""
    core = lab_a == 0
    return bool(np.array_equal(lab_a == 0, lab_b == 0) and np.array_equal(cid_a[core], cid_b[core]))
