import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
_ALL = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))
GOLDEN = [n for n in _ALL if not n.startswith("spheres")]  # triangle fixtures
SPHERE_GOLDEN = [n for n in _ALL if n.startswith("spheres")]  # user-primitive fixtures
SPHERE_UV_TOL = 2e-6  # |u|, |v| difference allowed on the GPU (atan2f / acosf vs the host's libm)


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


def load_sphere_golden(name: str) -> dict:
    import oracle

    d = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    d["nodes"] = d["nodes"].reshape(-1).view(oracle.NODE_DTYPE)
    d["sphere_hits"] = d["sphere_hits"].reshape(-1).view(oracle.SPHERE_HIT_DTYPE)
    return d


def sphere_hit_mismatches(a: np.ndarray, b: np.ndarray, uv_tol: float = 0.0) -> np.ndarray:
    """Indices where two sphere-hit arrays differ: prim, or the bits of t
    and the normal, or u / v by more than uv_tol."""
    a = np.asarray(a)
    b = np.asarray(b)
    au, bu = a.view(np.uint32).reshape(-1, 8), b.view(np.uint32).reshape(-1, 8)
    diff = np.any(au[:, [0, 1, 4, 5, 6]] != bu[:, [0, 1, 4, 5, 6]], axis=1)
    if uv_tol == 0.0:
        diff |= np.any(au[:, 2:4] != bu[:, 2:4], axis=1)
    else:
        du = np.abs(a["u"].astype(np.float64) - b["u"]) > uv_tol
        dv = np.abs(a["v"].astype(np.float64) - b["v"]) > uv_tol
        diff |= du | dv
    return np.nonzero(diff)[0]


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
