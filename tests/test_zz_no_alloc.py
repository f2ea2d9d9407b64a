"""The allocation-free build entry point, called through the C ABI.

lbvh_build_triangles_noalloc serves callers that cannot allocate device
memory where they build a BVH (a frame loop that sizes everything at start-up,
a plugin inside a host application that owns the GPU memory budget, a process
whose memory another allocator holds). It keeps its scratch in one fixed array
inside the library. This file is collected last, so a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import lbvh_gb300 as lb
from lbvh_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(tris, nodes, status, stream):
    L = _lib.lib()
    return L.lbvh_build_triangles_noalloc(
        ctypes.c_void_p(tris.data_ptr()), tris.shape[0],
        ctypes.c_void_p(nodes.data_ptr()),
        ctypes.c_void_p(status.data_ptr()) if status is not None else None,
        ctypes.c_void_p(stream))


def test_noalloc_build_matches_allocating_build(lib_built, port):
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    ctx = lb.Context(0, stream)
    status = torch.full((1,), 0xFFFF, dtype=torch.int32, device=dev)
    # calls in a row: two full-size soups (the tree's global phase and its
    # arrival slots run at this size), then smaller ones; each call reuses
    # (and must fully reset) the scratch the previous one left behind
    for n, seed in [(_lib.NOALLOC_MAX_PRIMS, 71), (_lib.NOALLOC_MAX_PRIMS, 74), (3_001, 72), (2, 73)]:
        tris_h = scenes.soup(n, seed)
        tris = torch.from_numpy(tris_h).to(dev)
        nodes = torch.empty(((n - 1) * 8,), dtype=torch.int32, device=dev)
        status.fill_(0xFFFF)
        assert _noalloc(tris, nodes, status, stream) == _lib.LBVH_OK
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        want = lb.Builder(ctx)(tris).nodes()  # the allocating entry point
        got = nodes.cpu().numpy().view(lb.NODE_DTYPE)
        assert got.tobytes() == want.tobytes(), n  # build parity is bit-exact
        assert got.tobytes() == port.build(tris_h, 8).tobytes(), n  # and equal to the oracle


def test_noalloc_without_status_word(lib_built, port):
    """d_status may be NULL: the build still runs and is still exact."""
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for n, seed in [(50_000, 75), (50_000, 76)]:
        tris_h = scenes.soup(n, seed)
        tris = torch.from_numpy(tris_h).to(dev)
        nodes = torch.empty(((n - 1) * 8,), dtype=torch.int32, device=dev)
        assert _noalloc(tris, nodes, None, stream) == _lib.LBVH_OK
        torch.cuda.synchronize()
        assert nodes.cpu().numpy().view(lb.NODE_DTYPE).tobytes() == port.build(tris_h, 8).tobytes(), seed


def test_noalloc_replays_in_a_captured_graph(lib_built, port):
    """One call captured into a CUDA graph and replayed on new triangles in
    the same buffer gives each soup's nodes: every replay clears the scratch
    words it reads, so nothing of an earlier replay is taken as current."""
    dev = torch.device("cuda", 0)
    n = _lib.NOALLOC_MAX_PRIMS
    tris = torch.from_numpy(scenes.soup(n, 80)).to(dev)
    nodes = torch.empty(((n - 1) * 8,), dtype=torch.int32, device=dev)
    status = torch.zeros((1,), dtype=torch.int32, device=dev)
    s = torch.cuda.Stream(dev)
    torch.cuda.synchronize()
    assert _noalloc(tris, nodes, status, s.cuda_stream) == _lib.LBVH_OK  # the device's set-up, outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        rc = _noalloc(tris, nodes, status, s.cuda_stream)
    assert rc == _lib.LBVH_OK
    for seed in (81, 82):
        t = scenes.soup(n, seed)
        tris.copy_(torch.from_numpy(t))
        status.fill_(0xFFFF)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        assert nodes.cpu().numpy().view(lb.NODE_DTYPE).tobytes() == port.build(t, 8).tobytes(), seed


def test_noalloc_rejects_what_it_cannot_serve(lib_built):
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    n = _lib.NOALLOC_MAX_PRIMS + 1
    tris = torch.zeros((n, 12), dtype=torch.float32, device=dev)
    nodes = torch.empty(((n - 1) * 8,), dtype=torch.int32, device=dev)
    assert _noalloc(tris, nodes, None, stream) == _lib.LBVH_ERR_INVALID_ARG
    one = torch.zeros((1, 12), dtype=torch.float32, device=dev)
    assert _noalloc(one, nodes, None, stream) == _lib.LBVH_ERR_INVALID_ARG
    host = torch.zeros((16, 12), dtype=torch.float32)
    assert _noalloc(host, nodes, None, stream) == _lib.LBVH_ERR_INVALID_ARG
    torch.cuda.synchronize()
