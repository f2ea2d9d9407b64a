import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
GOLDEN = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_golden(name: str) -> dict:
    import oracle

    d = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    d["nodes"] = d["nodes"].reshape(-1).view(oracle.NODE_DTYPE)
    d["sorted_leaf_nodes"] = d["sorted_leaf_nodes"].reshape(-1).view(oracle.NODE_DTYPE)
    if "hits" in d:
        d["hits"] = d["hits"].reshape(-1).view(oracle.HIT_DTYPE)
        d["sorted_leaf_hits"] = d["sorted_leaf_hits"].reshape(-1).view(oracle.HIT_DTYPE)
    if "user_box_nodes" in d:
        d["user_box_nodes"] = d["user_box_nodes"].reshape(-1).view(oracle.NODE_DTYPE)
    return d


@pytest.fixture(scope="session")
def port():
    import oracle

    return oracle.port()


@pytest.fixture(scope="session")
def lib_built():
    """The CUDA library, built in-tree if missing (nvcc cross-compiles)."""
    from lbvh_gb300 import _build

    return _build.build()


def hit_mismatches(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Indices where two hit arrays differ: prim ids, or (for hits) the bits
    of t, u, v."""
    a = np.asarray(a).view(np.uint32).reshape(-1, 4)
    b = np.asarray(b).view(np.uint32).reshape(-1, 4)
    hit = a[:, 0] != 0xFFFFFFFF
    diff = (a[:, 0] != b[:, 0]) | (hit & np.any(a[:, 1:] != b[:, 1:], axis=1))
    return np.nonzero(diff)[0]


def nodes_equal(a: np.ndarray, b: np.ndarray) -> bool:
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()
