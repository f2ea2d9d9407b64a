"""The request server: every result of a mixed, overlapping request stream
equals the same request run alone through the plain API (bit for bit), with
coalesced small builds/traces, several streams, and LRU eviction under a
small HBM budget."""
import numpy as np
import pytest

import lbvh_gb300 as lb
from lbvh_gb300 import scenes
from lbvh_gb300.serve import Server, run_plain, scene_bytes
from conftest import hit_mismatches

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _stream(n=160, n_scenes=20, hi=150_000, seed=4):
    return scenes.served_requests(n, 2000.0, seed, n_scenes=n_scenes, lo=300, hi=hi, ray_lo=1000,
                                  ray_hi=120_000)


def _serve(reqs, **kw):
    with Server(**kw) as srv:
        futs = [srv.submit(kind, scene, data) for _, kind, scene, data in reqs]
        results = [f.result(timeout=120) for f in futs]
        stats = {"coalesced": srv.coalesced, "evictions": srv.evictions}
    return results, stats


def test_mixed_stream_matches_plain_path(lib_built):
    assert torch.cuda.is_available()
    reqs = _stream()
    plain = run_plain([(0.0, k, s, d) for _, k, s, d in reqs])
    got, stats = _serve(reqs, slots=4)
    assert stats["coalesced"] > 0  # the initial small builds were batched
    for (_, kind, scene, _), (want, _), res in zip(reqs, plain, got):
        if kind == "trace":
            assert hit_mismatches(res, want).size == 0, scene
        else:
            assert res is None


def test_eviction_under_a_small_budget(lib_built):
    # room for four scenes: each new build evicts the least recently used
    # scene without queued work; the scenes still resident trace correctly
    meshes = [scenes.torus_mesh(40_000, 50 + k) for k in range(10)]
    budget = 4 * scene_bytes(meshes[0].shape[0]) + 1024
    with Server(slots=2, hbm_budget=budget, batch_max_tris=0, host_budget=0) as srv:
        for k, m in enumerate(meshes):
            srv.submit("build", k, m).result(timeout=60)
        assert srv.evictions >= 6
        assert sorted(srv.resident) == [6, 7, 8, 9]
        rays = scenes.incoherent_rays(meshes[9], 20_000, 1)
        got = srv.submit("trace", 9, rays).result(timeout=60)
        with pytest.raises(KeyError):
            srv.submit("trace", 0, rays).result(timeout=60)  # evicted
    want = run_plain([(0.0, "build", 9, meshes[9]), (0.0, "trace", 9, rays)])[1][0]
    assert hit_mismatches(got, want).size == 0


def test_trace_of_unknown_scene_fails_cleanly(lib_built):
    with Server(slots=1) as srv:
        f = srv.submit("trace", 12345, scenes.pinhole_rays(4, 4))
        with pytest.raises(KeyError):
            f.result(timeout=30)
        t = scenes.soup(100, 1)
        srv.submit("build", 1, t).result(timeout=30)
        hits = srv.submit("trace", 1, scenes.incoherent_rays(t, 500, 2)).result(timeout=30)
        assert hits.shape == (500,)


def test_rejected_requests_leave_the_server_usable(lib_built):
    t = scenes.soup(1000, 3)
    with Server(slots=2, hbm_budget=scene_bytes(1000) + 1024) as srv:
        srv.submit("build", 1, t).result(timeout=30)
        with pytest.raises(ValueError):  # a refit keeps the triangle count
            srv.submit("refit", 1, t[:999]).result(timeout=30)
        hits = srv.submit("trace", 1, np.zeros((0, 8), np.float32)).result(timeout=30)
        assert hits.shape == (0,)
        with pytest.raises(MemoryError):  # larger than the whole budget
            srv.submit("build", 2, scenes.soup(5000, 4)).result(timeout=30)
        srv.submit("build", 3, t).result(timeout=30)
        rays = scenes.incoherent_rays(t, 300, 5)
        got = srv.submit("trace", 3, rays).result(timeout=30)
    want = run_plain([(0.0, "build", 3, t), (0.0, "trace", 3, rays)])[1][0]
    assert hit_mismatches(got, want).size == 0


def test_evicted_scenes_are_dumped_and_reloaded(lib_built):
    """With a host budget, an evicted scene's tree goes to host memory and
    its next trace loads it back: the hits equal a fresh build's, and a refit
    of a reloaded scene works as on any resident tree. When the host budget
    is full, the least recently used dump is dropped: that scene is gone."""
    import time

    meshes = [scenes.torus_mesh(30_000, 60 + k) for k in range(8)]
    each = scene_bytes(meshes[0].shape[0])
    dump = 32 * (meshes[0].shape[0] - 1) + 48 * meshes[0].shape[0]
    rays = [scenes.incoherent_rays(m, 5_000, 70 + k) for k, m in enumerate(meshes)]
    moved = scenes.jitter(meshes[3], 5, 0.01)
    with Server(slots=2, hbm_budget=3 * each + 1024, batch_max_tris=0, host_budget=4 * dump + 1024) as srv:
        for k, m in enumerate(meshes):
            srv.submit("build", k, m).result(timeout=60)
        deadline = time.time() + 30
        while srv.spills < 5 and time.time() < deadline:  # dumps are copied out asynchronously
            time.sleep(0.01)
        assert srv.evictions == 5 and srv.spills == 5 and srv.spilled == 4
        with pytest.raises(KeyError):  # the oldest dump fell out of the host budget
            srv.submit("trace", 0, rays[0]).result(timeout=60)
        got1 = srv.submit("trace", 1, rays[1]).result(timeout=60)  # loaded back
        assert srv.reloads == 1
        got3 = srv.submit("trace", 3, rays[3]).result(timeout=60)
        srv.submit("refit", 3, moved).result(timeout=60)
        got3b = srv.submit("trace", 3, rays[3]).result(timeout=60)
        assert srv.reloads == 2
    want1 = run_plain([(0.0, "build", 1, meshes[1]), (0.0, "trace", 1, rays[1])])[1][0]
    want3 = run_plain([(0.0, "build", 3, meshes[3]), (0.0, "trace", 3, rays[3]),
                       (0.0, "refit", 3, moved), (0.0, "trace", 3, rays[3])])
    assert hit_mismatches(got1, want1).size == 0
    assert hit_mismatches(got3, want3[1][0]).size == 0
    assert hit_mismatches(got3b, want3[3][0]).size == 0


def test_page_locked_request_buffers(lib_built):
    """Requests whose triangles, rays and hit buffers are page-locked host
    memory (pinned tensors' storage, and cudaHostRegister'd numpy arrays)
    give the plain path's results."""
    t = scenes.soup(20_000, 61)
    rays = scenes.incoherent_rays(t, 50_000, 62)
    want = run_plain([(0.0, "build", 0, t), (0.0, "trace", 0, rays)])[1][0]
    pinned_t = torch.from_numpy(t).pin_memory()
    pinned_r = torch.from_numpy(rays).pin_memory()
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32).pin_memory()
    reg = np.ascontiguousarray(rays.copy())
    reg_hits = np.empty(rays.shape[0], lb.HIT_DTYPE)
    cudart = torch.cuda.cudart()
    for a in (reg, reg_hits):
        assert int(getattr(r := cudart.cudaHostRegister(a.ctypes.data, a.nbytes, 0), "value", r)) == 0
    try:
        with Server(slots=2) as srv:
            srv.submit("build", 0, pinned_t.numpy()).result(timeout=120)
            got = srv.submit("trace", 0, pinned_r.numpy(), out=hits.numpy().view(lb.HIT_DTYPE).reshape(-1)).result(timeout=120)
            assert hit_mismatches(got, want).size == 0
            got = srv.submit("trace", 0, reg, out=reg_hits).result(timeout=120)
            assert hit_mismatches(got, want).size == 0
    finally:
        for a in (reg, reg_hits):
            cudart.cudaHostUnregister(a.ctypes.data)


def test_injected_allocation_failures(lib_built):
    """Allocation failures injected on the host: the failing requests raise
    MemoryError, the HBM budget they held comes back, a scene whose rebuild
    failed keeps its previous tree, and the server goes on serving with the
    plain path's results."""
    t1, t2 = scenes.soup(30_000, 91), scenes.soup(30_000, 92)
    rays = scenes.incoherent_rays(t1, 4_000, 93)
    with Server(slots=2, batch_max_tris=0) as srv:
        srv.submit("build", 1, t1).result(timeout=60)
        before = srv.submit("trace", 1, rays).result(timeout=60)
        used = srv.used
        srv.inject_alloc_failures(1)
        with pytest.raises(MemoryError):
            srv.submit("build", 1, t2).result(timeout=60)  # the rebuild fails ...
        assert srv.used == used
        kept = srv.submit("trace", 1, rays).result(timeout=60)  # ... and the old tree stays
        assert hit_mismatches(kept, before).size == 0
        srv.inject_alloc_failures(1)
        with pytest.raises(MemoryError):
            srv.submit("build", 2, t2).result(timeout=60)
        assert srv.used == used and 2 not in srv.resident
        with pytest.raises(KeyError):
            srv.submit("trace", 2, rays).result(timeout=60)
        srv.submit("build", 2, t2).result(timeout=60)  # nothing injected any more
        got = srv.submit("trace", 2, rays).result(timeout=60)
    want = run_plain([(0.0, "build", 2, t2), (0.0, "trace", 2, rays)])[1][0]
    assert hit_mismatches(got, want).size == 0


def test_injected_failure_of_a_coalesced_build(lib_built):
    """Small builds coalesced into one batched build share one allocation:
    an injected failure fails those requests only; the others are built."""
    meshes = [scenes.soup(2_000 + 100 * k, 100 + k) for k in range(6)]
    with Server(slots=1) as srv:
        srv.inject_alloc_failures(1)
        futs = [srv.submit("build", k, m) for k, m in enumerate(meshes)]
        failed = []
        for k, f in enumerate(futs):
            try:
                f.result(timeout=60)
            except MemoryError:
                failed.append(k)
        assert failed  # the first allocation failed
        assert sorted(srv.resident) == [k for k in range(6) if k not in failed]
        assert srv.used == sum(scene_bytes(meshes[k].shape[0]) for k in srv.resident)
        for k in failed:  # a later build of the same scene succeeds
            srv.submit("build", k, meshes[k]).result(timeout=60)
        assert sorted(srv.resident) == list(range(6))


def test_cancelled_request_never_runs(lib_built):
    """A trace queued behind a long rebuild of its scene is cancelled before
    it starts: it raises CancelledError, the next trace runs normally."""
    from concurrent.futures import CancelledError

    big = scenes.soup_large(4_000_000, 94)
    rays = scenes.incoherent_rays(big, 2_000, 95)
    with Server(slots=1) as srv:
        srv.submit("build", 1, big)
        f = srv.submit("trace", 1, rays)  # waits for the build (same scene)
        srv.cancel(f)
        with pytest.raises(CancelledError):
            f.result(timeout=120)
        assert srv.cancelled == 1
        got = srv.submit("trace", 1, rays).result(timeout=120)
    want = run_plain([(0.0, "build", 1, big), (0.0, "trace", 1, rays)])[1][0]
    assert hit_mismatches(got, want).size == 0


def test_requests_expire_in_the_queue(lib_built):
    """With max_queue_s, requests that wait longer than that behind other
    work fail with TimeoutError; the others complete, and an idle server
    starts new requests at once."""
    soups = [scenes.soup_large(3_000_000, 96 + k) for k in range(6)]
    with Server(slots=1, max_queue_s=0.002, batch_max_tris=0) as srv:
        futs = [srv.submit("build", k, s) for k, s in enumerate(soups)]
        ok = expired = 0
        for f in futs:
            try:
                f.result(timeout=120)
                ok += 1
            except TimeoutError:
                expired += 1
        assert expired >= 1 and ok + expired == len(soups)
        assert srv.expired == expired
        t = scenes.soup(1_000, 97)
        srv.submit("build", 100, t).result(timeout=60)
        assert 100 in srv.resident
