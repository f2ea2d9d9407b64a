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


def test_room_config_is_identical_for_identical_rays():
    """Both arms build the step's config from their own bounce rays; equal
    rays give an equal config (the digest covers every ray of the step)."""
    tris = scenes.soup(100, 1)
    prim = scenes.pinhole_rays(8, 8)
    bounce = prim[::2].copy()
    a = bench.room_config(tris, prim, bounce, 1)
    b = bench.room_config(tris.copy(), prim.copy(), bounce.copy(), 1)
    assert a == b and a["rays_per_step"] == 96
    bounce[0, 0] += 1.0
    assert bench.room_config(tris, prim, bounce, 1)["rays_sha1"] != a["rays_sha1"]


def test_final_line_stays_short():
    """The final JSON line keeps the contract's keys and one-line summaries
    of the extra sections, short enough to survive a log tail."""
    import json

    served = {"throughput_ratio": 6.5, "server": {"p99_ms": 36.5}, "plain": {"p99_ms": 290.7}, "results_equal": True}
    line = {"metric": bench.METRIC, "value": 55.0, "unit": "Mrays/s", "n_gpus": 1, "steps": 20, "warmup": 5,
            "ms_per_step": 75.3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": bench.room_config(scenes.soup(10, 1), scenes.pinhole_rays(4, 4),
                                                             scenes.pinhole_rays(2, 2), 1),
            "build": {"ms": 0.1, "mprims_s": 2000.0}, "trace": {"ms": 75.0, "mrays_s": 55.0,
                                                                "primary_hit_fraction": 0.99},
            "build_16m": {"ms": 1.03, "mprims_s": 15500.0, "refit_ms": 0.6, "triangles": 16000000,
                          "roofline": {"frac": 0.6, "achieved": 4000.0}},
            "config1": {"value": 3900.0, "ms_per_step": 0.53, "build_ms": 0.07, "trace_ms": 0.46, "workload": "t"},
            "batched": {"graph_step_ms": 628.1, "plain_step_ms": 26441.0, "speedup_vs_plain": 42.1,
                        "sorted_leaves": {"step_ms": 12.9}, "tuning": {"x": 1}},
            "served": {"mix": served, "small": served},
            "roofline": {"bound": "hbm", "kernel": "lbvh build, 16M-triangle soup (all build kernels)",
                         "achieved": 4070.1, "peak": 6697.8, "unit": "GB/s", "frac": 0.6077, "bytes_per_prim": 264,
                         "traffic": 2762219008, "traffic_scope": "DRAM bytes of one whole build (all kernels), ncu",
                         "peak_kind": "measured"},
            "trace_profile": {"issue_slots_busy": 0.7, "simt_threads_per_instruction": 16.0, "l1_hit_rate": 0.8,
                              "l2_hit_rate": 0.9, "warps_active_of_max": 0.45, "source": "profiles/x.md"},
            "cpu_baseline": {"value": 0.6, "unit": "Mrays/s", "cores": 16, "kind": "reference",
                             "lib": "oracle/_ref/libref.so", "sample": "build of all 262267 triangles + every 16th "
                                                                       "primary and bounce ray (258858) per step, 3 steps"},
            "e2e": {"value": 50.0, "unit": "Mrays/s", "ms_per_step": 80.0, "h2d_bytes_per_step": 145125000,
                    "d2h_bytes_per_step": 66267664, "transfer": "triangles copied; rays read and hits written in "
                                                                "place in page-locked host memory"},
            "gpu_launches": 220, "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 10}}
    out = bench.summary_line(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in out, k
    assert out["served"]["small"]["ratio"] == 6.5 and out["build_16m"]["frac"] == 0.6
    assert len(json.dumps(out)) < 3000
