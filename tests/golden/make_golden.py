"""Generates the golden fixtures in this folder from the UNMODIFIED reference.

Run where the reference's files are available (they are not needed
afterwards):

    sh oracle/stage_ref.sh [REF_SRC]    # copies them into baseline/_ref
    make -C oracle                      # builds oracle/_ref/libref.so
    python tests/golden/make_golden.py  # writes tests/golden/*.npz

Each fixture stores its inputs (so the GPU host, which has no reference tree,
can replay them) and the reference's outputs through oracle/ref_shim.cpp:
centroid bounds, per-primitive Morton codes, the sorted code sequence, the
stable sort permutation, the node array, and closest hits for a ray set.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from lbvh_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF_DIR = oracle.ref_dir()  # $LBVH_REF_DIR, else the copy staged in baseline/_ref


def edge_rays(tris: np.ndarray, nodes: np.ndarray, seed: int) -> np.ndarray:
    """Axis-parallel rays (dir components exactly 0, both signs), rays whose
    origins sit exactly on node-box planes, and a few random rays."""
    lo, hi = scenes.scene_box(tris)
    c = 0.5 * (lo + hi)
    out = []
    grid = np.linspace(-1.2, 1.2, 9)
    for axis in range(3):
        for sgn in (1.0, -1.0):
            for a in grid:
                for b in grid:
                    o = c.copy()
                    o[axis] = (hi[axis] + 0.5) if sgn < 0 else (lo[axis] - 0.5)
                    o[(axis + 1) % 3] = c[(axis + 1) % 3] + a * 0.5 * (hi - lo)[(axis + 1) % 3]
                    o[(axis + 2) % 3] = c[(axis + 2) % 3] + b * 0.5 * (hi - lo)[(axis + 2) % 3]
                    d = np.zeros(3)
                    d[axis] = sgn
                    out.append(np.r_[o, d, 0.0, np.inf])
    # origins on the planes of node boxes, pointing at the scene centre or
    # along an axis (exercises 0 * inf = NaN slabs in the box test)
    k = min(len(nodes), 64)
    idx = np.linspace(0, len(nodes) - 1, k).astype(int)
    for j, i in enumerate(idx):
        b_lo = nodes["lo"][i].astype(np.float64)
        b_hi = nodes["hi"][i].astype(np.float64)
        o = np.where(np.arange(3) == j % 3, b_lo, 0.5 * (b_lo + b_hi))
        d = c - o
        if j % 2:
            d = np.zeros(3)
            d[(j + 1) % 3] = 1.0 if j % 4 == 1 else -1.0
        out.append(np.r_[o, d, 0.0, np.inf])
        out.append(np.r_[b_hi, -(b_hi - c), 0.0, np.inf])
    # rays aimed at triangle centroids, vertices and edge midpoints (tied and
    # grazing hits between neighbouring triangles)
    verts = scenes.triangle_vertices(tris).astype(np.float64)
    pick = np.linspace(0, len(tris) - 1, min(len(tris), 48)).astype(int)
    org = scenes.incoherent_rays(tris, 3 * len(pick), seed + 100)[:, 0:3].astype(np.float64)
    for j, i in enumerate(pick):
        for q, target in enumerate((verts[i].mean(0), verts[i][0], 0.5 * (verts[i][1] + verts[i][2]))):
            o = org[3 * j + q]
            out.append(np.r_[o, target - o, 0.0, np.inf])
    r = np.array(out, np.float32)
    rnd = scenes.incoherent_rays(tris, 256, seed)
    rnd[::4, 6] = 0.25  # some nonzero tmin / finite tmax
    rnd[1::4, 7] = 1.0
    return np.concatenate([r, rnd])


def dump(name: str, tris: np.ndarray, rays: np.ndarray | None, R, boxes: np.ndarray | None = None):
    rec = {"tris": tris}
    rec["boxes"] = R.tri_boxes(tris)
    rec["bounds"] = R.centroid_bounds(tris, 4)
    codes, scodes, perm = R.curve(tris, 4)
    rec["codes"], rec["sorted_codes"], rec["stable_perm"] = codes, scodes, perm
    nodes = R.build(tris, 4)
    rec["nodes"] = nodes.view(np.uint8).reshape(-1, 32)
    if rays is not None:
        rec["rays"] = rays
        rec["hits"] = R.trace(nodes, tris, rays, 4).view(np.uint8).reshape(-1, 16)
    # sorted-leaf mode: the unmodified builder run on triangles pre-permuted
    # by the stable sort permutation
    pt = tris[perm]
    pn = R.build(pt, 4)
    rec["sorted_leaf_nodes"] = pn.view(np.uint8).reshape(-1, 32)
    if rays is not None:
        rec["sorted_leaf_hits"] = R.trace(pn, pt, rays, 4).view(np.uint8).reshape(-1, 16)
    if boxes is not None:
        rec["user_boxes"] = boxes
        rec["user_box_nodes"] = R.build_boxes(boxes, 4).view(np.uint8).reshape(-1, 32)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(f"{name}: n={tris.shape[0]} rays={0 if rays is None else rays.shape[0]}")


def dump_spheres(name: str, spheres: np.ndarray, rays: np.ndarray, R):
    """User primitives: the example program's spheres, its sphere_to_box
    converter (centre +- radius, float32), the reference builder over those
    boxes, and its traverser with the example's intersector."""
    from lbvh_gb300.api import sphere_boxes

    boxes = sphere_boxes(spheres)
    nodes = R.build_boxes(boxes, 4)
    hits = R.trace_spheres(nodes, spheres, rays, 4)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), spheres=spheres, sphere_boxes=boxes,
                        nodes=nodes.view(np.uint8).reshape(-1, 32), rays=rays,
                        sphere_hits=hits.view(np.uint8).reshape(-1, 32))
    print(f"{name}: n={spheres.shape[0]} rays={rays.shape[0]} hit={np.mean(hits['prim'] != oracle.MISS):.3f}")


def main():
    oracle.build_libs(REF_DIR)
    R = oracle.ref()
    if R is None:
        raise SystemExit(f"reference not built (looked in {REF_DIR})")

    # config 0: 968-triangle soup, 64x64 pinhole rays at (0,0,3), 60 deg
    t = scenes.soup(968, seed=1)
    dump("soup968", t, scenes.pinhole_rays(64, 64), R)

    # the reference's shipped meshes, loaded by its own tinyobj path
    for mesh in ("monkey", "teapot"):
        path = os.path.join(REF_DIR, "models", mesh + ".obj")
        mt = R.load_obj(path)
        lo, hi = scenes.scene_box(mt)
        c = 0.5 * (lo + hi)
        eye = c + np.array([0.0, 0.0, 1.6 * float(np.max(hi - lo))])
        dump(mesh, mt, scenes.pinhole_rays(48, 48, eye=eye, target=c), R)

    # config-1 geometry: torus + ground plane, primary + incoherent rays
    ts = scenes.torus_scene(seed=11)
    rays = np.concatenate([scenes.pinhole_rays(48, 48), scenes.incoherent_rays(ts, 2048, 3)])
    dump("torus8320", ts, rays, R)

    # edge cases
    v2 = scenes.soup_vertices(2, 5)
    t2 = scenes.make_triangles(v2)
    dump("n2", t2, edge_rays(t2, R.build(t2, 1), 1), R)
    t3 = scenes.soup(3, 6)
    dump("n3", t3, edge_rays(t3, R.build(t3, 1), 2), R)
    # all-equal triangles: every code equal, the clz(i ^ j) + 32 tie path
    te = scenes.make_triangles(np.tile(scenes.soup_vertices(1, 7), (1000, 1)))
    dump("all_equal1000", te, edge_rays(te, R.build(te, 1), 3), R)
    # heavy duplicate codes: centroids snapped to a coarse 6^3 lattice
    vq = scenes.soup_vertices(4000, 8)
    cen = vq.reshape(-1, 3, 3).mean(1)
    snapped = np.round(cen * 2.5) / 2.5
    vq = (vq.reshape(-1, 3, 3) - cen[:, None] + snapped[:, None]).reshape(-1, 9)
    tq = scenes.make_triangles(vq)
    dump("dups4000", tq, edge_rays(tq, R.build(tq, 1), 4), R)
    # signed zeros: coordinates that are exactly +0 or -0, axis-aligned
    # triangles, and degenerate (zero-area / collinear / point) triangles
    g = np.linspace(-1, 1, 5).astype(np.float32)
    gz = []
    for x in g:
        for y in g:
            for s in (0.0, -0.0):
                gz.append([x, y, s, x + 0.25, y, s, x, y + 0.25, s])
                gz.append([s, x, y, s, x + 0.25, y, s, x, y + 0.25])
    gz = np.array(gz, np.float32)
    zero = np.zeros((40, 9), np.float32)
    zero[1::2] = -0.0
    degen = scenes.soup_vertices(60, 9)
    degen[0:20, 3:6] = degen[0:20, 0:3]                          # a == b
    degen[20:40, 6:9] = 2 * degen[20:40, 3:6] - degen[20:40, 0:3]  # collinear
    degen[40:60, 3:9] = np.tile(degen[40:60, 0:3], 2)            # a point
    tz = scenes.make_triangles(np.concatenate([gz, zero, degen]))
    dump("zeros_degenerate", tz, edge_rays(tz, R.build(tz, 1), 5), R)
    # user boxes (the sphere example's converter: centre +- radius)
    sp = scenes.uniform(12, 0, 4 * 500).reshape(500, 4)
    cen = (sp[:, :3] * 10 - 5).astype(np.float32)
    rad = (0.05 + 0.3 * sp[:, 3:]).astype(np.float32)
    boxes = np.concatenate([cen - rad, cen + rad], 1).astype(np.float32)
    dump("soup2000_boxes", scenes.soup(2000, 13), None, R, boxes=boxes)

    # user primitives with the example program's intersector: its own three
    # spheres under its camera, and a 2,000-sphere scene with rays from
    # inside and outside the spheres (negative roots included)
    dump_spheres("spheres_example", scenes.example_spheres(), scenes.example_camera_rays(96, 54), R)
    sph = scenes.sphere_scene(2000, 21)
    lo, hi = sph[:, 1:].min(0), sph[:, 1:].max(0)
    rays = np.concatenate([scenes.random_rays_in_box(lo, hi, 3000, 22), scenes.pinhole_rays(40, 40, eye=(0, 0, 9))])
    dump_spheres("spheres2000", sph, rays, R)


if __name__ == "__main__":
    main()
