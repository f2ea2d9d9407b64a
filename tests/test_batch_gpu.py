"""Batched build + trace of many meshes in one launch each: every mesh's node
block and hits equal the oracle (pinned to the reference) run on that mesh
alone, bit for bit."""
import numpy as np
import pytest

import lbvh_gb300 as lb
from lbvh_gb300 import _lib, scenes
from conftest import hit_mismatches, load_golden, nodes_equal

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx(lib_built):
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return lb.Context()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def make_batch(sizes, seed):
    meshes = [scenes.soup(n, seed * 1000 + i) for i, n in enumerate(sizes)]
    for name in ("teapot", "dups4000", "all_equal1000", "n2"):
        meshes.append(load_golden(name)["tris"])
    off = np.zeros(len(meshes) + 1, np.uint32)
    off[1:] = np.cumsum([m.shape[0] for m in meshes])
    return meshes, np.concatenate(meshes), off


@pytest.mark.parametrize("threads", [256, 512, 1024])
def test_batch_build_matches_oracle(ctx, port, threads):
    ctx.set_param(_lib.PARAM_BATCH_THREADS, threads)
    try:
        sizes = [2, 3, 5, 64, 1000, 4095, 4096, 4097, 20000, 65536]
        meshes, tris, off = make_batch(sizes, threads)
        for src_t, src_o in ((tris, off), (dev(tris), dev(off.view(np.int32)))):
            b = lb.Batch(ctx).build(src_t, src_o)
            all_nodes = b.nodes()
            for k, m in enumerate(meshes):
                assert nodes_equal(b.mesh_nodes(k, all_nodes), port.build(m, 8)), (threads, k, m.shape[0])
    finally:
        ctx.set_param(_lib.PARAM_BATCH_THREADS, 512)


@pytest.mark.parametrize("bits,items", [(4, 4), (6, 4), (6, 8), (8, 8), (4, 8)])
@pytest.mark.parametrize("sorted_leaves", [False, True])
def test_batch_radix_width_and_keys_per_thread(ctx, port, bits, items, sorted_leaves):
    """Every radix width (4, 6, 8 bits: an even and an odd number of passes)
    and keys-per-thread setting of the CTA-local sort gives every mesh the
    plain build's node block (and, with sorted leaves, its leaf order)."""
    ctx.set_param(_lib.PARAM_BATCH_RADIX_BITS, bits)
    ctx.set_param(_lib.PARAM_BATCH_KEYS_PER_THREAD, items)
    try:
        meshes, tris, off = make_batch([2, 3, 64, 1000, 4097, 20000, 65536], bits * 10 + items)
        b = lb.Batch(ctx).build(dev(tris), off, sorted_leaves=sorted_leaves)
        all_nodes = b.nodes()
        for k, m in enumerate(meshes):
            if sorted_leaves:
                perm = port.curve(m, 8)[2]
                want = port.build(m[perm], 8)
            else:
                want = port.build(m, 8)
            assert nodes_equal(b.mesh_nodes(k, all_nodes), want), (bits, items, k, m.shape[0])
    finally:
        ctx.set_param(_lib.PARAM_BATCH_RADIX_BITS, 8)
        ctx.set_param(_lib.PARAM_BATCH_KEYS_PER_THREAD, 4)
    with pytest.raises(ValueError):
        ctx.set_param(_lib.PARAM_BATCH_RADIX_BITS, 5)
    with pytest.raises(ValueError):
        ctx.set_param(_lib.PARAM_BATCH_KEYS_PER_THREAD, 6)


@pytest.mark.parametrize("leaf_batch", [1, 8])
def test_batch_trace_matches_oracle(ctx, port, leaf_batch):
    ctx.set_param(_lib.PARAM_TRACE_LEAF_BATCH, leaf_batch)
    try:
        _batch_trace_matches_oracle(ctx, port)
    finally:
        ctx.set_param(_lib.PARAM_TRACE_LEAF_BATCH, 1)


def _batch_trace_matches_oracle(ctx, port):
    meshes, tris, off = make_batch([2, 17, 500, 3000, 40000], 7)
    b = lb.Batch(ctx).build(dev(tris), off)
    rays, roff = [], [0]
    for k, m in enumerate(meshes):
        r = scenes.incoherent_rays(m, 700 + 100 * k, k)
        rays.append(r)
        roff.append(roff[-1] + r.shape[0])
    rays_all = np.concatenate(rays)
    roff = np.array(roff, np.uint32)
    got = lb.hits_view(b.trace(dev(rays_all), dev(roff.view(np.int32))))
    got_h = b.trace(rays_all, roff)
    assert got.tobytes() == got_h.tobytes()
    all_nodes = b.nodes()
    for k, m in enumerate(meshes):
        want = port.trace(b.mesh_nodes(k, all_nodes), m, rays[k], 4)
        seg = got[roff[k] : roff[k + 1]]
        assert hit_mismatches(seg, want).size == 0, k


def test_batch_rejects_bad_offsets(ctx):
    tris = scenes.soup(100, 1)
    with pytest.raises(ValueError):
        lb.Batch(ctx).build(tris, np.array([0, 1, 100], np.uint32))  # a one-triangle mesh
    with pytest.raises(ValueError):
        lb.Batch(ctx).build(tris, np.array([0, 50, 99], np.uint32))  # does not end at the total
    # device offsets are checked on the device and reported at the next sync
    bad = dev(np.array([0, 60, 59, 100], np.uint32).view(np.int32))
    lb.Batch(ctx).build(dev(tris), bad)
    with pytest.raises(lb.LbvhError):
        ctx.synchronize()
    ok = lb.Batch(ctx).build(dev(tris), np.array([0, 30, 100], np.uint32))
    assert ok.nodes().size == 98


@pytest.mark.parametrize("threads", [256, 1024])
def test_sorted_leaf_batch_matches_plain_sorted_leaf_builds(ctx, threads):
    """Sorted-leaf batches: each mesh's node block equals the plain
    sorted-leaf build of that mesh (itself pinned to the reference builder
    run on the stably pre-sorted triangles), and the batched trace's hits,
    with input-order triangle ids, equal the plain sorted-leaf trace's."""
    ctx.set_param(_lib.PARAM_BATCH_THREADS, threads)
    try:
        meshes, tris, off = make_batch([2, 3, 64, 1000, 4097, 30000], 11 + threads)
        b = lb.Batch(ctx).build(dev(tris), off, sorted_leaves=True)
        all_nodes = b.nodes()
        rays, roff, want = [], [0], []
        for k, m in enumerate(meshes):
            plain = lb.Builder(ctx, sorted_leaves=True)(m)
            assert nodes_equal(b.mesh_nodes(k, all_nodes), plain.nodes()), (threads, k)
            r = scenes.incoherent_rays(m, 500, 40 + k)
            rays.append(r)
            roff.append(roff[-1] + r.shape[0])
            want.append(lb.Traverser(plain)(r))
        got = lb.hits_view(b.trace(dev(np.concatenate(rays)), dev(np.array(roff, np.uint32).view(np.int32))))
        assert hit_mismatches(got, np.concatenate(want)).size == 0
    finally:
        ctx.set_param(_lib.PARAM_BATCH_THREADS, 512)
