"""The CPU oracle (oracle/lbvh_oracle.cpp) pinned against outputs of the
unmodified reference: the committed golden fixtures everywhere, and the
reference itself (oracle/_ref) where it was built."""
import numpy as np
import pytest

import oracle
from lbvh_gb300 import scenes
from conftest import (GOLDEN, SPHERE_GOLDEN, hit_mismatches, load_golden, load_sphere_golden, nodes_equal,
                      sphere_hit_mismatches)


@pytest.mark.parametrize("name", GOLDEN)
def test_port_matches_golden_build(port, name):
    g = load_golden(name)
    t = g["tris"]
    assert np.array_equal(port.tri_boxes(t).view(np.uint32), g["boxes"].view(np.uint32))
    for threads in (1, 3, 8):
        assert np.array_equal(port.centroid_bounds(t, threads).view(np.uint32), g["bounds"].view(np.uint32))
        codes, sc, perm = port.curve(t, threads)
        assert np.array_equal(codes, g["codes"])
        assert np.array_equal(sc, g["sorted_codes"])
        assert np.array_equal(perm, g["stable_perm"])
        assert nodes_equal(port.build(t, threads), g["nodes"])
    assert nodes_equal(port.build(t[g["stable_perm"]], 4), g["sorted_leaf_nodes"])
    if "user_boxes" in g:
        assert nodes_equal(port.build_boxes(g["user_boxes"], 4), g["user_box_nodes"])


@pytest.mark.parametrize("name", [n for n in GOLDEN if n != "soup2000_boxes"])
def test_port_matches_golden_trace(port, name):
    g = load_golden(name)
    hits = port.trace(g["nodes"], g["tris"], g["rays"], threads=4)
    assert hit_mismatches(hits, g["hits"]).size == 0
    pt = g["tris"][g["stable_perm"]]
    hits = port.trace(g["sorted_leaf_nodes"], pt, g["rays"], threads=2)
    assert hit_mismatches(hits, g["sorted_leaf_hits"]).size == 0


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_trees_satisfy_reference_invariants(port, name):
    # check_bvh + check_volumes, lbvh_test.cpp:369-518
    g = load_golden(name)
    assert port.check_bvh(g["nodes"]) == 0
    assert port.check_bvh(g["sorted_leaf_nodes"]) == 0


def test_check_bvh_catches_planted_errors(port):
    g = load_golden("soup968")
    nodes = g["nodes"].copy()
    assert port.check_bvh(nodes) == 0
    bad = nodes.copy()
    bad["left"][5] = bad["left"][6]  # a node referenced twice / a leaf lost
    assert port.check_bvh(bad) > 0
    bad = nodes.copy()
    i = int(np.nonzero((nodes["left"] & oracle.LEAF_BIT) == 0)[0][0])
    child = nodes["left"][i]
    bad["lo"][child] -= 10.0  # child box grows beyond its parent
    assert port.check_bvh(bad) > 0


def test_numpy_triangles_match_golden(port):
    g = load_golden("soup968")
    v = scenes.soup_vertices(968, seed=1)  # the vertices soup968 was made from
    assert np.array_equal(scenes.make_triangles(v).view(np.uint32), g["tris"].view(np.uint32))
    assert np.array_equal(port.make_triangles(v).view(np.uint32), g["tris"].view(np.uint32))


def test_port_refit_equals_fresh_fit(port):
    # refit over the same topology with unmoved primitives reproduces the build
    g = load_golden("teapot")
    nodes = g["nodes"].copy()
    nodes["lo"] = 0
    nodes["hi"] = 0
    assert nodes_equal(port.refit(nodes, g["tris"]), g["nodes"])


REF = oracle.ref()


@pytest.mark.skipif(REF is None, reason="reference not built on this machine")
@pytest.mark.parametrize("n,seed", [(2, 1), (5, 2), (100, 3), (4097, 4), (20000, 5)])
def test_port_matches_reference_random(port, n, seed):
    t = scenes.soup(n, seed)
    for threads in (1, 8):
        assert nodes_equal(port.build(t, threads), REF.build(t, threads))
        for a, b in zip(port.curve(t, threads), REF.curve(t, threads)):
            assert np.array_equal(a, b)
    nodes = REF.build(t, 4)
    rays = np.concatenate([scenes.pinhole_rays(32, 32), scenes.incoherent_rays(t, 1024, seed)])
    assert hit_mismatches(port.trace(nodes, t, rays, 4), REF.trace(nodes, t, rays, 4)).size == 0


@pytest.mark.skipif(REF is None, reason="reference not built on this machine")
def test_port_matches_reference_boxes():
    b = scenes.uniform(3, 0, 6 * 3000).reshape(3000, 6).astype(np.float32)
    boxes = np.concatenate([np.minimum(b[:, :3], b[:, 3:]), np.maximum(b[:, :3], b[:, 3:])], 1)
    assert nodes_equal(oracle.port().build_boxes(boxes, 4), REF.build_boxes(boxes, 4))


@pytest.mark.skipif(REF is None, reason="reference not built on this machine")
def test_port_matches_reference_at_gpu_test_sizes(port):
    """The port against the reference at the sizes the GPU suite compares
    the library with the port: a 300,007-triangle soup, the 262,267-triangle
    room scene, and the 1.6M-triangle soup with 18,000 equal triangles."""
    for t, m in ((scenes.soup(300_007, 300_007), 1024), (scenes.room_scene(seed=2), 4096)):
        nodes = REF.build(t, 8)
        assert nodes_equal(port.build(t, 8), nodes)
        rays = scenes.incoherent_rays(t, m, 7)
        assert hit_mismatches(port.trace(nodes, t, rays, 8), REF.trace(nodes, t, rays, 8)).size == 0
    t = scenes.soup_large(1_600_000, seed=90)
    t[:18_000] = t[0]
    assert nodes_equal(port.build(t, 16), REF.build(t, 16))


@pytest.mark.skipif(REF is None, reason="reference not built on this machine")
def test_port_matches_reference_16m_soup(port):
    """The roofline workload, the 16M-triangle soup, built by the port and
    by the reference (about 15 s with the generation)."""
    t = scenes.soup_large(16_000_000, seed=16)
    assert nodes_equal(port.build(t, 16), REF.build(t, 16))


@pytest.mark.skipif(REF is None, reason="reference not built on this machine")
def test_port_matches_reference_extreme_inputs(port):
    """The inputs of the GPU suite's edge-case traversal and signed-zero
    tests, through the port and the reference: far-out triangles (boxes
    beyond 2^60), nearly axis-parallel rays, -0.0 direction components, far
    origins, and vertex coordinates that are +0.0 and -0.0 in turn."""
    t = scenes.soup(3000, seed=12)
    far = scenes.soup(8, seed=13) * np.float32(1e30)
    t = np.concatenate([t, far]).astype(np.float32)
    nodes = REF.build(t, 4)
    assert nodes_equal(port.build(t, 4), nodes)
    rays = scenes.incoherent_rays(t[:3000], 20_000, 14)
    rays[::7, 3] = np.float32(1e-30)
    rays[1::11, 4] = np.float32(-0.0)
    rays[2::13, 0:3] *= np.float32(1e25)
    assert hit_mismatches(port.trace(nodes, t, rays, 4), REF.trace(nodes, t, rays, 4)).size == 0
    rng = np.random.default_rng(15)
    v = rng.uniform(-1, 1, (4000, 9)).astype(np.float32)
    zero = rng.random(v.shape) < 0.3
    v[zero] = np.where(rng.random(zero.sum()) < 0.5, np.float32(0.0), np.float32(-0.0))
    tz = scenes.make_triangles(v)
    assert nodes_equal(port.build(tz, 4), REF.build(tz, 4))
    for a, b in zip(port.curve(tz, 4), REF.curve(tz, 4)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", SPHERE_GOLDEN)
def test_port_matches_golden_spheres(port, name):
    """User primitives: the example program's spheres, boxes from its
    converter, the reference's builder and its traverser with the example's
    intersector; the port agrees bit for bit (uv included: same host libm)."""
    from lbvh_gb300.api import sphere_boxes

    g = load_sphere_golden(name)
    boxes = sphere_boxes(g["spheres"])
    assert np.array_equal(boxes.view(np.uint32), g["sphere_boxes"].view(np.uint32))
    assert nodes_equal(port.build_boxes(boxes, 3), g["nodes"])
    for threads in (1, 5):
        hits = port.trace_spheres(g["nodes"], g["spheres"], g["rays"], threads)
        assert sphere_hit_mismatches(hits, g["sphere_hits"]).size == 0
