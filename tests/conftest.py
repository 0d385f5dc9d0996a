import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "fd-weno-eulerequation_gb300", "python"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_fixture(path):
    z = np.load(path)
    out = {k: z[k] for k in z.files}
    out["meta"] = json.loads(str(out["meta"]))
    return out


def fixture_paths(prefix=""):
    return sorted(glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def fixture_id(path):
    return os.path.basename(path)[:-4]


def assert_same(a, b, what=""):
    """Bitwise-equal values (== semantics, so +0 and -0 agree)."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
    if bad.any():
        idx = np.argwhere(bad)[0]
        rel = np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))
        pytest.fail(f"{what}: {bad.sum()} values differ, first at {tuple(idx)}: "
                    f"{a[tuple(idx)]!r} vs {b[tuple(idx)]!r}, max rel {rel:.3e}")


@pytest.fixture
def golden():
    return load_fixture
