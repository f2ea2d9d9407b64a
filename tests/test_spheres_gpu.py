"""User primitives on the GPU: a BVH built from the boxes of the reference
example program's spheres (its sphere_to_box converter run on the host) and
traced with the example's sphere intersector on the device. The hit sphere,
t and the normal must equal the reference's bit for bit; u and v, which come
from atan2 / acos, within SPHERE_UV_TOL."""
import numpy as np
import pytest

import lbvh_gb300 as lb
from lbvh_gb300 import scenes
from conftest import SPHERE_GOLDEN, SPHERE_UV_TOL, load_sphere_golden, nodes_equal, sphere_hit_mismatches

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("name", SPHERE_GOLDEN)
def test_sphere_trace_matches_reference(lib_built, name):
    g = load_sphere_golden(name)
    boxes = lb.sphere_boxes(g["spheres"])
    bvh = lb.Builder()(boxes, converter=lb.BOXES)
    assert nodes_equal(bvh.nodes(), g["nodes"])
    hits = lb.SphereTraverser(bvh, g["spheres"])(g["rays"])
    assert sphere_hit_mismatches(hits, g["sphere_hits"], SPHERE_UV_TOL).size == 0
    # device-resident spheres, rays and hits take the asynchronous path
    dev = torch.device("cuda")
    sph = torch.from_numpy(g["spheres"]).to(dev)
    rays = torch.from_numpy(g["rays"]).to(dev)
    out = lb.SphereTraverser(bvh, sph)(rays)
    torch.cuda.synchronize()
    dh = out.cpu().numpy().view(lb.SPHERE_HIT_DTYPE).reshape(-1)
    assert sphere_hit_mismatches(dh, hits).size == 0


def test_sphere_trace_matches_oracle_on_a_larger_scene(lib_built, port):
    sph = scenes.sphere_scene(50_000, 31, extent=20.0)
    lo, hi = sph[:, 1:].min(0), sph[:, 1:].max(0)
    rays = scenes.random_rays_in_box(lo, hi, 40_000, 32)
    boxes = lb.sphere_boxes(sph)
    bvh = lb.Builder()(boxes, converter=lb.BOXES)
    nodes = bvh.nodes()
    assert nodes_equal(nodes, port.build_boxes(boxes, 8))
    got = lb.SphereTraverser(bvh, sph)(rays)
    want = port.trace_spheres(nodes, sph, rays, 8)
    assert sphere_hit_mismatches(got, want, SPHERE_UV_TOL).size == 0
    assert np.mean(got["prim"] != lb.MISS) > 0.05


def test_sphere_trace_rejects_sorted_leaves_and_bad_counts(lib_built):
    sph = scenes.sphere_scene(100, 33)
    boxes = lb.sphere_boxes(sph)
    with pytest.raises(ValueError):
        lb.SphereTraverser(lb.Builder(sorted_leaves=True)(boxes, converter=lb.BOXES), sph)
    bvh = lb.Builder()(boxes, converter=lb.BOXES)
    with pytest.raises(ValueError):
        lb.SphereTraverser(bvh, sph[:50])
    assert lb.SphereTraverser(bvh, sph)(np.zeros((0, 8), np.float32)).shape == (0,)
