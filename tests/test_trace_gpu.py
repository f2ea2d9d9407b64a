"""GPU closest-hit parity: hits (primitive id and the bits of t, u, v) and the
per-ray box/triangle test counts against the reference's golden outputs and
the pinned CPU oracle. The arithmetic and visiting order are the reference's,
so the expected mismatch count is zero (the acceptance bar is >= 99.999% of
ids equal with t within 1e-6 relative)."""
import numpy as np
import pytest

import lbvh_gb300 as lb
from lbvh_gb300 import _lib, scenes
from conftest import nodes_equal, GOLDEN, hit_mismatches, load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx(lib_built):
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return lb.Context()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def assert_hits_equal(got, want):
    bad = hit_mismatches(got, want)
    assert bad.size == 0, f"{bad.size} of {len(want)} rays differ, first {bad[:8]}"
    hit = want["prim"] != lb.MISS
    assert np.all(np.isinf(got["t"][~hit]))


@pytest.mark.parametrize("name", [n for n in GOLDEN if n != "soup2000_boxes"])
def test_trace_matches_golden(ctx, name):
    g = load_golden(name)
    bvh = lb.Builder(ctx)(dev(g["tris"]))
    assert_hits_equal(lb.Traverser(bvh)(g["rays"]), g["hits"])
    got = lb.hits_view(lb.Traverser(bvh)(dev(g["rays"])))
    assert_hits_equal(got, g["hits"])
    # sorted-leaf mode reports original primitive ids
    sl = lb.Builder(ctx, sorted_leaves=True)(dev(g["tris"]))
    want = g["sorted_leaf_hits"].copy()
    hit = want["prim"] != lb.MISS
    want["prim"][hit] = g["stable_perm"][want["prim"][hit]]
    assert_hits_equal(lb.Traverser(sl)(g["rays"]), want)


def test_config0_full_pinhole(ctx, port):
    # 968-triangle random soup, 256 x 256 pinhole rays from (0, 0, 3), 60 deg
    t = scenes.soup(968, seed=1)
    rays = scenes.pinhole_rays(256, 256)
    bvh = lb.Builder(ctx)(dev(t))
    nodes = port.build(t, 8)
    want, nb, nt = port.trace(nodes, t, rays, 16, counts=True)
    got, gb, gt = lb.Traverser(bvh)(rays, counts=True)
    assert_hits_equal(got, want)
    assert np.array_equal(gb, nb) and np.array_equal(gt, nt)


def test_config1_torus_primary_and_incoherent(ctx, port):
    # 6,320-triangle torus + 2,000-triangle plane; 1024^2 primary and 1M
    # incoherent rays
    t = scenes.torus_scene(seed=11)
    rays = np.concatenate([scenes.pinhole_rays(1024, 1024), scenes.incoherent_rays(t, 1 << 20, 3)])
    bvh = lb.Builder(ctx)(dev(t))
    want = port.trace(port.build(t, 8), t, rays, 16)
    got = lb.hits_view(lb.Traverser(bvh)(dev(rays)))
    assert_hits_equal(got, want)


def test_config2_room_primary_and_diffuse_bounce(ctx, port):
    # 262,267-triangle clustered room; 1920 x 1080 primary rays from inside
    # the room and one cosine-weighted diffuse bounce per hit, the bounce rays
    # made from the oracle's hits so both sides trace the same rays
    t = scenes.room_scene(seed=21)
    bvh = lb.Builder(ctx)(dev(t))
    nodes = port.build(t, 16)
    assert nodes_equal(bvh.nodes(), nodes)
    prim = scenes.pinhole_rays(1920, 1080, eye=(0.0, 3.0, 9.0), target=(0.0, 2.0, 0.0))
    want = port.trace(nodes, t, prim, 16)
    assert_hits_equal(lb.hits_view(lb.Traverser(bvh)(dev(prim))), want)
    assert np.mean(want["prim"] != lb.MISS) > 0.5
    bounce = scenes.diffuse_bounce(prim, want, t, seed=22)
    want_b = port.trace(nodes, t, bounce, 16)
    assert_hits_equal(lb.hits_view(lb.Traverser(bvh)(dev(bounce))), want_b)


def test_edge_rays_random_soup(ctx, port):
    # axis-parallel rays (0 * inf slabs), rays from box planes, finite tmax
    t = scenes.soup(5000, seed=5)
    nodes = port.build(t, 8)
    lo, hi = scenes.scene_box(t)
    rays = []
    for axis in range(3):
        for s in (1.0, -1.0):
            g = np.linspace(-1.0, 1.0, 33)
            a, b = np.meshgrid(g, g)
            o = np.zeros((a.size, 3))
            o[:, axis] = -2.0 * s
            o[:, (axis + 1) % 3] = a.reshape(-1)
            o[:, (axis + 2) % 3] = b.reshape(-1)
            d = np.zeros_like(o)
            d[:, axis] = s
            r = np.zeros((a.size, 8))
            r[:, 0:3], r[:, 3:6], r[:, 7] = o, d, np.inf
            rays.append(r)
    r = np.concatenate(rays).astype(np.float32)
    r[::3, 7] = 2.0
    r[1::5, 6] = 1.5
    bvh = lb.Builder(ctx)(dev(t))
    assert_hits_equal(lb.Traverser(bvh)(r), port.trace(nodes, t, r, 8))


def test_extreme_coordinates_and_directions(ctx, port):
    """Box coordinates beyond 2^60 switch the traversal to the reference's
    exact ternary min/max (the fast fminf/fmaxf slab path needs every slab
    value finite), and so do rays with a direction component below 2^-60 in
    magnitude; hits stay bit-identical."""
    t = scenes.soup(3000, seed=12)
    far = scenes.soup(8, seed=13) * np.float32(1e30)  # a few triangles far out
    t = np.concatenate([t, far]).astype(np.float32)
    nodes = port.build(t, 8)
    bvh = lb.Builder(ctx)(dev(t))
    assert nodes_equal(bvh.nodes(), nodes)
    rays = scenes.incoherent_rays(t[:3000], 20_000, 14)
    rays[::7, 3] = np.float32(1e-30)   # nearly axis-parallel rays
    rays[1::11, 4] = np.float32(-0.0)
    rays[2::13, 0:3] *= np.float32(1e25)  # origins far out
    assert_hits_equal(lb.hits_view(lb.Traverser(bvh)(dev(rays))), port.trace(nodes, t, rays, 8))


def test_signed_zero_ties_in_boxes(ctx, port):
    """Triangles whose vertex coordinates are +0.0 and -0.0 in turn: every
    min/max tie between the two zeros resolves as the reference's folds do
    (bounds, leaf boxes, node boxes compared bit for bit)."""
    rng = np.random.default_rng(15)
    v = rng.uniform(-1, 1, (4000, 9)).astype(np.float32)
    zero = rng.random(v.shape) < 0.3
    v[zero] = np.where(rng.random(zero.sum()) < 0.5, np.float32(0.0), np.float32(-0.0))
    t = scenes.make_triangles(v)
    bvh = lb.Builder(ctx, keep_curve=True)(dev(t))
    assert nodes_equal(bvh.nodes(), port.build(t, 8))
    assert nodes_equal(lb.Builder(ctx)(dev(t)).nodes(), port.build(t, 8))
    assert np.array_equal(bvh.curve()[3].view(np.uint32), port.centroid_bounds(t, 8).view(np.uint32))


def test_user_box_bvh_has_no_triangle_traverser(ctx):
    b = lb.Builder(ctx)(np.zeros((4, 6), np.float32), converter=lb.BOXES)
    with pytest.raises(ValueError):
        lb.Traverser(b)


@pytest.mark.parametrize("name", ["soup968", "teapot", "dups4000"])
def test_trace_imported_reference_nodes(ctx, name):
    # a node array made by the reference itself, traced on the GPU
    g = load_golden(name)
    bvh = lb.BVH.from_nodes(g["nodes"], g["tris"], ctx)
    assert_hits_equal(lb.Traverser(bvh)(g["rays"]), g["hits"])
    bvh = lb.BVH.from_nodes(dev(g["nodes"].view(np.uint8)), dev(g["tris"]), ctx)
    assert_hits_equal(lb.Traverser(bvh)(g["rays"]), g["hits"])


def test_import_rejects_malformed_trees(ctx):
    g = load_golden("soup968")
    bad = g["nodes"].copy()
    bad["left"][3] = bad["left"][4]  # a node referenced twice, another lost
    with pytest.raises(lb.LbvhError):
        lb.BVH.from_nodes(bad, g["tris"], ctx)
    bad = g["nodes"].copy()
    bad["right"][7] = 5000  # an internal index out of range
    with pytest.raises(lb.LbvhError):
        lb.BVH.from_nodes(bad, g["tris"], ctx)
    # the context stays usable
    ok = lb.BVH.from_nodes(g["nodes"], g["tris"], ctx)
    assert_hits_equal(lb.Traverser(ok)(g["rays"]), g["hits"])


def test_host_pointer_traces_match_device_traces(ctx):
    """Traces given host rays and/or host hit buffers go through chunked,
    overlapped copies once they are large; every combination returns the
    same hits as the all-device call (sizes straddle the chunking)."""
    t = scenes.torus_scene(seed=11)
    bvh = lb.Builder(ctx)(dev(t))
    ctx.set_param(_lib.PARAM_TRACE_CHUNK, 1 << 18)  # several chunks, with a remainder
    for m in (1000, (1 << 19) - 1, (1 << 19) + 12345, 1 << 21):
        rays = scenes.incoherent_rays(t, m, m % 97)
        ref = lb.hits_view(lb.Traverser(bvh)(dev(rays)))
        host_host = lb.Traverser(bvh)(rays)
        pinned = torch.from_numpy(rays).pin_memory()
        host_dev = lb.hits_view(lb.Traverser(bvh)(pinned, out=torch.empty((m, 4), device="cuda")))
        dev_host = np.empty(m, lb.HIT_DTYPE)
        lb.Traverser(bvh)(dev(rays), out=dev_host)
        ctx.synchronize()
        for got in (host_host, host_dev, dev_host):
            assert got.tobytes() == ref.tobytes(), m
    ctx.set_param(_lib.PARAM_TRACE_CHUNK, 1 << 20)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_pinned_traces_in_place_match_device_traces(ctx, mode):
    """Page-locked host rays and hit buffers are copied (mode 0), or the
    rays are read in place (1) and the hits written in place too (2, each
    warp writing its batches of 32 hits from shared memory); every mode and
    mix returns the device call's hits, for counts that are not multiples of
    32 and ones that span many batches per warp."""
    t = scenes.torus_scene(seed=11)
    bvh = lb.Builder(ctx)(dev(t))
    ctx.set_param(_lib.PARAM_TRACE_IN_PLACE, mode)
    try:
        for m in (1, 1000, 12345, (1 << 20) + 7):
            rays = scenes.incoherent_rays(t, m, m % 89)
            ref = lb.hits_view(lb.Traverser(bvh)(dev(rays))).tobytes()
            rays_p = torch.from_numpy(rays).pin_memory()
            hits_p = torch.empty((m, 4), dtype=torch.float32).pin_memory()
            lb.Traverser(bvh)(rays_p, out=hits_p)
            assert lb.hits_view(hits_p).tobytes() == ref, (mode, m)
            hits_p.fill_(-1.0)
            lb.Traverser(bvh)(dev(rays), out=hits_p)  # device rays, pinned hits
            assert lb.hits_view(hits_p).tobytes() == ref, (mode, m)
            got = lb.Traverser(bvh)(rays_p, out=torch.empty((m, 4), device="cuda"))  # pinned rays, device hits
            assert lb.hits_view(got).tobytes() == ref, (mode, m)
        # pinned buffers that are not 16-byte aligned are copied instead
        m = 4097
        rays = scenes.incoherent_rays(t, m, 5)
        ref = lb.hits_view(lb.Traverser(bvh)(dev(rays))).tobytes()
        rays_p = torch.empty(8 * m + 1, dtype=torch.float32).pin_memory()
        rays_p[1:] = torch.from_numpy(rays.reshape(-1))
        hits_p = torch.empty(4 * m + 1, dtype=torch.float32).pin_memory()
        lb.Traverser(bvh)(rays_p[1:].view(m, 8), out=hits_p[1:].view(m, 4))
        assert lb.hits_view(hits_p[1:].view(m, 4)).tobytes() == ref, mode
    finally:
        ctx.set_param(_lib.PARAM_TRACE_IN_PLACE, 2)


@pytest.mark.parametrize("leaf_batch", [1, 4, 32])
def test_leaf_batch_settings_match(ctx, port, leaf_batch):
    """Every setting of the traversal's leaf batching gives the reference's
    hits and per-ray box / triangle test counts (each ray keeps the
    reference's visit, test and cull order): the golden fixtures, the small
    config in full, and a slice of the large room's primary rays."""
    from lbvh_gb300 import _lib

    c = lb.Context()
    c.set_param(_lib.PARAM_TRACE_LEAF_BATCH, leaf_batch)
    for name in [n for n in GOLDEN if n != "soup2000_boxes"]:
        g = load_golden(name)
        got = lb.hits_view(lb.Traverser(lb.Builder(c)(dev(g["tris"])))(dev(g["rays"])))
        assert_hits_equal(got, g["hits"])
    t = scenes.soup(968, seed=1)
    rays = scenes.pinhole_rays(256, 256)
    nodes = port.build(t, 8)
    want, nb, nt = port.trace(nodes, t, rays, 16, counts=True)
    got, gb, gt = lb.Traverser(lb.Builder(c)(dev(t)))(rays, counts=True)
    assert_hits_equal(got, want)
    assert np.array_equal(gb, nb) and np.array_equal(gt, nt)
    room = scenes.room_scene(seed=21)
    prim = np.ascontiguousarray(scenes.pinhole_rays(1920, 1080, eye=(0.0, 3.0, 9.0), target=(0.0, 2.0, 0.0))[::37])
    want, nb, nt = port.trace(port.build(room, 16), room, prim, 16, counts=True)
    got, gb, gt = lb.Traverser(lb.Builder(c)(dev(room)))(prim, counts=True)
    assert_hits_equal(got, want)
    assert np.array_equal(gb, nb) and np.array_equal(gt, nt)
    with pytest.raises(ValueError):
        c.set_param(_lib.PARAM_TRACE_LEAF_BATCH, 0)


@pytest.mark.parametrize("leaf_batch", [1, 8])
def test_sorted_ray_order_gives_the_same_hits(ctx, port, leaf_batch):
    """With LBVH_PARAM_TRACE_RAY_ORDER the rays are traversed in sorted order
    (origin cell, then direction cell), and every hit and per-ray count
    still lands in its ray's slot: the reference's hits for the room's
    primary and diffuse bounce rays (device, host and page-locked buffers),
    the torus config's incoherent rays, and sizes on either side of the
    4,096-ray minimum."""
    c = lb.Context()
    c.set_param(_lib.PARAM_TRACE_LEAF_BATCH, leaf_batch)
    c.set_param(_lib.PARAM_TRACE_RAY_ORDER, 1)
    room = scenes.room_scene(seed=21)
    nodes = port.build(room, 16)
    prim = np.ascontiguousarray(scenes.pinhole_rays(1920, 1080, eye=(0.0, 3.0, 9.0), target=(0.0, 2.0, 0.0))[::23])
    bvh = lb.Builder(c)(dev(room))
    trav = lb.Traverser(bvh)
    want_p, nb, nt = port.trace(nodes, room, prim, 16, counts=True)
    assert_hits_equal(lb.hits_view(trav(dev(prim))), want_p)
    got, gb, gt = trav(prim, counts=True)
    assert_hits_equal(got, want_p)
    assert np.array_equal(gb, nb) and np.array_equal(gt, nt)
    bounce = scenes.diffuse_bounce(prim, want_p, room, seed=22)
    want_b = port.trace(nodes, room, bounce, 16)
    assert_hits_equal(lb.hits_view(trav(dev(bounce))), want_b)
    assert_hits_equal(trav(bounce), want_b)  # host rays and hits
    pinned = torch.from_numpy(bounce).pin_memory()
    assert_hits_equal(lb.hits_view(trav(pinned)), want_b)
    for m in (4095, 4096, 4097, 9999):
        assert_hits_equal(lb.hits_view(trav(dev(bounce[:m]))), want_b[:m])
    t = scenes.torus_scene(seed=11)
    rays = scenes.incoherent_rays(t, 1 << 16, 3)
    assert_hits_equal(lb.hits_view(lb.Traverser(lb.Builder(c)(dev(t)))(dev(rays))), port.trace(port.build(t, 8), t, rays, 16))
    with pytest.raises(ValueError):
        c.set_param(_lib.PARAM_TRACE_RAY_ORDER, 2)
