"""GPU build parity: the CUDA library against the reference's golden outputs
and against the pinned CPU oracle, bit for bit (Morton codes, sorted codes,
stable permutation, centroid bounds, node topology and node boxes)."""
import numpy as np
import pytest

import lbvh_gb300 as lb
from lbvh_gb300 import scenes
from conftest import GOLDEN, load_golden, nodes_equal

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx(lib_built):
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return lb.Context()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", GOLDEN)
def test_build_matches_golden(ctx, name):
    g = load_golden(name)
    for src in (g["tris"], dev(g["tris"])):  # host and device input
        bvh = lb.Builder(ctx, keep_curve=True)(src)
        codes, sc, perm, bounds = bvh.curve()
        assert np.array_equal(bounds.view(np.uint32), g["bounds"].view(np.uint32))
        assert np.array_equal(codes, g["codes"])
        assert np.array_equal(sc, g["sorted_codes"])
        assert np.array_equal(perm, g["stable_perm"])
        assert nodes_equal(bvh.nodes(), g["nodes"])
    # parity build without the curve (key-only sort path)
    assert nodes_equal(lb.Builder(ctx)(dev(g["tris"])).nodes(), g["nodes"])
    # sorted-leaf mode = the reference builder over Morton-ordered input
    assert nodes_equal(lb.Builder(ctx, sorted_leaves=True)(dev(g["tris"])).nodes(), g["sorted_leaf_nodes"])
    if "user_boxes" in g:
        b = lb.Builder(ctx)(dev(g["user_boxes"]), converter=lb.BOXES)
        assert nodes_equal(b.nodes(), g["user_box_nodes"])
        b = lb.Builder(ctx)(g["user_boxes"], converter=lambda x: x)  # host converter
        assert nodes_equal(b.nodes(), g["user_box_nodes"])


@pytest.mark.parametrize("n", [2, 3, 31, 1000, 4095, 4096, 4097, 8193, 20480, 20481, 65537, 300_007])
def test_build_matches_oracle_random(ctx, port, n):
    t = scenes.soup(n, seed=n)
    bvh = lb.Builder(ctx, keep_curve=True)(dev(t))
    codes, sc, perm = port.curve(t, 8)
    gc, gsc, gperm, gb = bvh.curve()
    assert np.array_equal(gc, codes)
    assert np.array_equal(gsc, sc)
    assert np.array_equal(gperm, perm)
    assert np.array_equal(gb.view(np.uint32), port.centroid_bounds(t, 8).view(np.uint32))
    ref_nodes = port.build(t, 8)
    assert nodes_equal(bvh.nodes(), ref_nodes)
    assert port.check_bvh(bvh.nodes()) == 0
    # keys-only build (one cluster launch up to 16,384 primitives, the
    # multi-kernel build above)
    assert nodes_equal(lb.Builder(ctx)(dev(t)).nodes(), ref_nodes)
    sl = lb.Builder(ctx, sorted_leaves=True)(dev(t))
    assert nodes_equal(sl.nodes(), port.build(t[perm], 8))


def test_rebuild_reuses_storage(ctx, port):
    # larger then smaller then larger builds into one handle and one context
    bvh = lb.BVH(ctx)
    b = lb.Builder(ctx)
    for n, seed in [(50_000, 1), (777, 2), (120_001, 3), (2, 4), (50_000, 5)]:
        t = scenes.soup(n, seed)
        b(dev(t), into=bvh)
        assert nodes_equal(bvh.nodes(), port.build(t, 8)), n


def test_duplicate_heavy_and_degenerate(ctx, port):
    # all centroids on a coarse lattice: long runs of equal codes
    v = scenes.soup_vertices(200_000, 9)
    c = v.reshape(-1, 3, 3).mean(1)
    v = (v.reshape(-1, 3, 3) - c[:, None] + (np.round(c * 3) / 3)[:, None]).reshape(-1, 9)
    t = scenes.make_triangles(v)
    assert nodes_equal(lb.Builder(ctx)(dev(t)).nodes(), port.build(t, 8))
    # every triangle identical: every code equal
    t = scenes.make_triangles(np.tile(scenes.soup_vertices(1, 3), (70_000, 1)))
    assert nodes_equal(lb.Builder(ctx)(dev(t)).nodes(), port.build(t, 8))


def test_make_triangles_kernel(ctx, port):
    v = scenes.soup_vertices(100_003, 21)
    want = port.make_triangles(v).view(np.uint32)
    assert np.array_equal(lb.make_triangles(v, ctx=ctx).view(np.uint32), want)
    got = lb.make_triangles(dev(v), ctx=ctx).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want)


@pytest.mark.parametrize("sorted_leaves", [False, True])
def test_refit_matches_oracle(ctx, port, sorted_leaves):
    t = scenes.soup(40_000, 31)
    bvh = lb.Builder(ctx, sorted_leaves=sorted_leaves)(dev(t))
    v = scenes.triangle_vertices(t).reshape(-1, 9).astype(np.float64)
    v += scenes.normal(31, 7, v.size).reshape(v.shape) * 0.01  # seeded jitter
    t2 = scenes.make_triangles(v.astype(np.float32))
    bvh.refit(dev(t2))
    nodes = bvh.nodes()
    if sorted_leaves:
        perm = port.curve(t, 8)[2]
        want = port.refit(port.build(t[perm], 8), t2[perm])
    else:
        want = port.refit(port.build(t, 8), t2)
    assert nodes_equal(nodes, want)
    # host-side refit input as well
    bvh.refit(t2)
    assert nodes_equal(bvh.nodes(), want)
    # a refit after another build on the same context (the codes are the BVH's own)
    lb.Builder(ctx)(dev(scenes.soup(50_000, 5)))
    bvh.refit(dev(t))
    want0 = port.build(t[perm], 8) if sorted_leaves else port.build(t, 8)
    assert nodes_equal(bvh.nodes(), want0)
    if not sorted_leaves:
        # a tree given as a node array has no codes: the refit walks its links
        loaded = lb.BVH.from_nodes(want0, t, ctx)
        loaded.refit(dev(t2))
        assert nodes_equal(loaded.nodes(), want)


@pytest.mark.parametrize("n", [300_000, 600_000, 2_000_000])
def test_large_refit_matches_oracle(ctx, port, n):
    """Refits of at least 2^19 primitives rerun the tree phase over the
    build's own sorted codes (smaller ones walk the node links); either way
    the result equals the oracle's topology-preserving fit."""
    t = scenes.soup(n, 41) if n <= 600_000 else scenes.soup_large(n, seed=41)
    bvh = lb.Builder(ctx)(dev(t))
    t2 = (t + np.float32(0.01)).astype(np.float32)
    bvh.refit(dev(t2))
    assert nodes_equal(bvh.nodes(), port.refit(port.build(t, 16), t2))
    if n == 600_000:  # sorted-leaf mode: the moved triangles are gathered into leaf order first
        sl = lb.Builder(ctx, sorted_leaves=True)(dev(t))
        sl.refit(dev(t2))
        perm = port.curve(t, 16)[2]
        assert nodes_equal(sl.nodes(), port.refit(port.build(t[perm], 16), t2[perm]))


def test_invalid_arguments_raise(ctx):
    with pytest.raises(ValueError):
        lb.Builder(ctx)(np.zeros((1, 12), np.float32))
    with pytest.raises(ValueError):
        lb.Builder(ctx)(np.zeros((5, 11), np.float32))
    with pytest.raises(ValueError):
        lb.Builder(ctx)(np.zeros((4, 12), np.float64))


@pytest.mark.parametrize("sorted_leaves", [False, True])
def test_lookback_wait_that_runs_out_reports_timeout(lib_built, port, sorted_leaves):
    """A radix-sort look-back wait that never sees its word gives up after
    the spin limit: the kernel returns, the build reports LBVH_ERR_TIMEOUT
    (no tree is built over the unsorted codes), and the same context then
    builds exactly again. The stall parameter makes every wait look for a
    tag no tile writes -- a flag that nothing sets."""
    from lbvh_gb300 import _lib

    c = lb.Context()
    t = scenes.soup(60_000, seed=81)
    c.set_param(_lib.PARAM_LOOKBACK_SPIN_LIMIT, 512)
    c.set_param(_lib.PARAM_TEST_LOOKBACK_STALL, 1)
    with pytest.raises(lb.LbvhError) as e:
        lb.Builder(c, sorted_leaves=sorted_leaves)(t)  # host input: the call returns finished
    assert e.value.status == _lib.LBVH_ERR_TIMEOUT
    c.set_param(_lib.PARAM_TEST_LOOKBACK_STALL, 0)
    with pytest.raises(ValueError):
        c.set_param(_lib.PARAM_LOOKBACK_SPIN_LIMIT, 0)
    c.set_param(_lib.PARAM_LOOKBACK_SPIN_LIMIT, 1 << 22)
    got = lb.Builder(c, sorted_leaves=sorted_leaves)(dev(t))
    c.synchronize()
    if sorted_leaves:
        perm = port.curve(t, 16)[2]
        assert nodes_equal(got.nodes(), port.build(t[perm], 16))
    else:
        assert nodes_equal(got.nodes(), port.build(t, 16))


@pytest.mark.parametrize("tile,bucket_min,bounds", [(1024, 1 << 30, 2), (4096, 1 << 30, 8), (0, 65536, 1),
                                                     (0, 65536, 16), (1024, 1 << 30, 16)])
def test_sort_and_bounds_parameters(lib_built, port, tile, bucket_min, bounds):
    """The plain build's tunable sort and bounds parameters (tile size of
    the keys-only sort, the bucket sort for builds from 65,536 primitives,
    the bounds pass's CTAs per SM) all give the reference's nodes: random
    soups around the tile and bucket boundaries, the clustered room and a
    duplicate-heavy input."""
    from lbvh_gb300 import _lib

    c = lb.Context()
    c.set_param(_lib.PARAM_SORT_TILE_KEYS, tile)
    c.set_param(_lib.PARAM_BUCKET_SORT_MIN, bucket_min)
    c.set_param(_lib.PARAM_BOUNDS_BLOCKS_PER_SM, bounds)
    cases = [scenes.soup(n, 90 + n % 7) for n in (2, 1000, 4097, 65536, 65537, 300_007)]
    cases.append(scenes.room_scene(seed=21))
    cases.append(load_golden("dups4000")["tris"])
    for t in cases:
        assert nodes_equal(lb.Builder(c)(dev(t)).nodes(), port.build(t, 16)), (tile, bucket_min, bounds, t.shape[0])
    for param, bad in ((_lib.PARAM_SORT_TILE_KEYS, 2048), (_lib.PARAM_BUCKET_SORT_MIN, 1000),
                       (_lib.PARAM_BOUNDS_BLOCKS_PER_SM, 17)):
        with pytest.raises(ValueError):
            c.set_param(param, bad)


@pytest.mark.parametrize("n", [2, 3, 1023, 1024, 1025, 2048, 7777, 8193, 16383, 16384, 16385])
def test_one_launch_build_matches_multi_kernel(lib_built, port, n):
    """Keys-only builds of up to 16,384 primitives run as one cluster launch
    (LBVH_PARAM_SMALL_BUILD_MAX); at 0 they take the multi-kernel build. Both
    give the reference's nodes, for triangles (host and device input) and for
    boxes, on random soups and on duplicate-heavy input."""
    from lbvh_gb300 import _lib

    one = lb.Context()
    multi = lb.Context()
    multi.set_param(_lib.PARAM_SMALL_BUILD_MAX, 0)
    for t in (scenes.soup(n, seed=n + 5), np.repeat(scenes.soup((n + 6) // 7, seed=n)[:, None], 7, 1)
              .reshape(-1, 12)[:n].copy()):
        if t.shape[0] < 2:
            continue
        want = port.build(t, 8)
        for c in (one, multi):
            assert nodes_equal(lb.Builder(c)(dev(t)).nodes(), want), (n, c is one)
            assert nodes_equal(lb.Builder(c)(t).nodes(), want), (n, c is one)
        boxes = port.tri_boxes(t)
        want_b = port.build_boxes(boxes, 8)
        for c in (one, multi):
            assert nodes_equal(lb.Builder(c)(dev(boxes), converter=lb.BOXES).nodes(), want_b), (n, c is one)
    torus = scenes.torus_scene(seed=3)
    assert nodes_equal(lb.Builder(one)(dev(torus)).nodes(), port.build(torus, 8))
    with pytest.raises(ValueError):
        one.set_param(_lib.PARAM_SMALL_BUILD_MAX, 16385)


@pytest.mark.parametrize("fused,merge_cap", [(0, 0), (1, 0), (0, 8)])
def test_tree_global_phase_fused_or_separate(lib_built, port, fused, merge_cap):
    """The nodes above the subtrees the local phase leaves at its CTA edges
    -- merged window by window in shared memory (one level up to 160 CTAs,
    two beyond), walked from the local phase's tail, or (a merge capacity of
    8 subtrees, too small for any window here) by the merge's fallback walk
    over the global slots -- are the reference's nodes, for builds and for
    refits that rerun the tree phase over the build's codes."""
    from lbvh_gb300 import _lib

    c = lb.Context()
    c.set_param(_lib.PARAM_TREE_WALK_FUSED, fused)
    c.set_param(_lib.PARAM_TEST_TREE_MERGE_CAP, merge_cap)
    for n in (20_000, 49_153, 300_007):
        t = scenes.soup(n, 70 + n % 5)
        assert nodes_equal(lb.Builder(c)(dev(t)).nodes(), port.build(t, 16)), (fused, n)
    room = scenes.room_scene(seed=21)
    assert nodes_equal(lb.Builder(c)(dev(room)).nodes(), port.build(room, 16))
    t = scenes.soup(600_000, 77)  # refits from 2^19 primitives rerun the tree phase
    b = lb.Builder(c)(dev(t))
    t2 = (t + np.float32(0.003)).astype(np.float32)
    b.refit(dev(t2))
    assert nodes_equal(b.nodes(), port.refit(port.build(t, 16), t2))
    with pytest.raises(ValueError):
        c.set_param(_lib.PARAM_TREE_WALK_FUSED, 2)
    with pytest.raises(ValueError):
        c.set_param(_lib.PARAM_TEST_TREE_MERGE_CAP, 3201)


def test_full_size_16m_build_parity(ctx, port):
    """The 16M-triangle random soup (the roofline workload) against the
    oracle, bit for bit, plus the reference's structural invariants."""
    n = 16_000_000
    t = scenes.soup_large(n, seed=16)
    d = dev(t)
    nodes = lb.Builder(ctx)(d).nodes()
    assert nodes_equal(nodes, port.build(t, 16))
    assert port.check_bvh(nodes) == 0


def test_dump_and_reload_round_trip(lib_built, tmp_path):
    """A BVH written with save() and read back with load() has the same
    nodes and primitives and traces to the same hits; a dump of a sorted-leaf
    tree is refused, and a corrupted node array is rejected on reload."""
    t = scenes.torus_scene(seed=12)
    bvh = lb.Builder()(t)
    p = tmp_path / "scene.npz"
    bvh.save(p)
    back = lb.BVH.load(p)
    assert np.array_equal(back.nodes().view(np.uint8), bvh.nodes().view(np.uint8))
    assert np.array_equal(back.primitives().view(np.uint32), t.view(np.uint32))
    rays = scenes.incoherent_rays(t, 4096, 13)
    a = lb.Traverser(bvh)(rays)
    b = lb.Traverser(back)(rays)
    assert a.tobytes() == b.tobytes()
    with pytest.raises(ValueError):
        lb.Builder(sorted_leaves=True)(t).save(tmp_path / "sorted.npz")
    d = dict(np.load(p))
    nodes = d["nodes"].reshape(-1).view(lb.NODE_DTYPE).copy()
    nodes["left"][5] = nodes["left"][6]  # two parents for one child
    d["nodes"] = nodes.view(np.uint8).reshape(-1, 32)
    np.savez(tmp_path / "bad.npz", **d)
    with pytest.raises(lb.LbvhError):
        lb.BVH.load(tmp_path / "bad.npz")


@pytest.mark.parametrize("kind,n", [("uniform", 1_600_000), ("dense_bucket", 1_600_000), ("over_bucket", 1_600_000),
                                    ("crowded", 1_600_000), ("all_equal", 1_600_000), ("over_bucket", 3_000_000)])
def test_large_builds_with_crowded_buckets_match_oracle(ctx, port, kind, n):
    """Keys-only builds of at least 1.5M primitives sort by buckets of the
    top 12 code bits when every bucket holds at most 20,480 codes and by the
    radix passes otherwise. A uniform soup and one with a bucket filled to
    19,543 codes (18,000 of them equal) take the first path; 1,000 more
    equal codes (20,542 in the bucket), a scene whose codes crowd one bucket,
    and one whose codes are all equal take the second. At 3M primitives the
    radix passes run on one wave of CTAs that loop over the tiles. All match
    the oracle."""
    if kind in ("uniform", "dense_bucket", "over_bucket"):
        t = scenes.soup_large(n, seed=90)
        if kind != "uniform":
            t[: 18_000 if kind == "dense_bucket" else 19_000] = t[0]
    elif kind == "crowded":
        t = scenes.soup_large(n, seed=91) * np.float32(1e-3)  # a tight cluster at the origin...
        t[:2000] *= np.float32(1e3)                           # ...and a few triangles spread wide
    else:
        t = np.tile(scenes.soup_large(1, seed=92), (n, 1))
    bvh = lb.Builder(ctx)(dev(t))
    assert nodes_equal(bvh.nodes(), port.build(t, 16))
