"""Host-side helpers of bench.py that need no GPU: the page-locked arena the
served benchmark carves request arrays and hit buffers from (here over a
plain host array), and the figures read from the committed ncu summaries."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402
import lbvh_gb300 as lb  # noqa: E402
from lbvh_gb300 import scenes  # noqa: E402


class _HostArena(bench._PinnedArena):
    """The arena's carving over ordinary host memory (no CUDA here)."""

    def __init__(self, nbytes):
        self._a = np.zeros(max(int(nbytes), 1), np.uint8)
        self._off = 0


def test_pinned_requests_keep_data_sharing_and_alignment(monkeypatch):
    monkeypatch.setattr(bench, "_PinnedArena", _HostArena)
    reqs = scenes.served_requests(300, 2000.0, 5, n_scenes=12, lo=1000, hi=20000, ray_lo=1000, ray_hi=20000)
    arena, moved = bench._pinned_requests(reqs)
    base, end = arena._a.ctypes.data, arena._a.ctypes.data + arena._a.size
    seen = {}
    for (at, kind, scene, d), (at2, kind2, scene2, d2) in zip(reqs, moved):
        assert (at, kind, scene) == (at2, kind2, scene2)
        assert d2.shape == d.shape and d2.dtype == d.dtype
        assert d2.tobytes() == d.tobytes()
        assert base <= d2.ctypes.data and d2.ctypes.data + d2.nbytes <= end  # inside the arena
        assert (d2.ctypes.data - base) % 16 == 0  # what an in-place trace needs (the arena is page-aligned)
        # a request array shared by several requests stays one array
        assert seen.setdefault(id(d), id(d2)) == id(d2)
    # every moved array, ray slices included, is a view of the one arena array
    pool_views = [d2 for (_, k, _, d), (_, _, _, d2) in zip(reqs, moved) if k == "trace"]
    owners = {id(bench._owner(v)) for v in pool_views}
    assert len(owners) == 1
    # both paths' hit buffers fit in what is left
    for _ in range(2):
        for _, kind, _, d in moved:
            if kind == "trace":
                h = arena.take(16 * d.shape[0]).view(lb.HIT_DTYPE)
                assert h.shape == (d.shape[0],) and (h.ctypes.data - base) % 256 == 0


def test_arena_refuses_to_overrun():
    a = _HostArena(1000)
    a.take(700)
    with pytest.raises(AssertionError):
        a.take(400)


def test_trace_profile_figures_come_from_the_committed_capture():
    p = bench.measured_profile("k_trace_tris", ("l1_hit_rate", "l2_hit_rate", "issue_slots_busy"))
    assert p is not None and set(p) == {"l1_hit_rate", "l2_hit_rate", "issue_slots_busy", "source"}
    assert all(0.0 < p[k] <= 1.0 for k in ("l1_hit_rate", "l2_hit_rate", "issue_slots_busy"))
    assert os.path.exists(os.path.join(ROOT, p["source"]))
    assert bench.measured_traffic("k_trace_tris", "dram_bytes_per_launch") > 0
    assert bench.measured_profile("no_such_kernel", ("l1_hit_rate",)) is None
