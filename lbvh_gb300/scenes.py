"""Seeded synthetic scenes and rays for the LBVH build/trace workloads.

Every generator is deterministic for a given seed: random numbers come from a
counter-based SplitMix64 hash of (seed, stream, index), so any slice of a scene
can be regenerated without generating the rest, and the same arrays feed the
CUDA path and the CPU oracle. Geometry is produced in float64 and rounded once
to float32.

Triangles are returned in the reference layout (tay10r/lbvh ``triangle<float>``,
lbvh.h:1959-1983): 12 float32 per triangle ``{p0, e0 = a - b, e1 = c - a,
normal = cross(e0, e1)}``, computed with one IEEE rounding per operation and no
fused multiply-add, exactly as the reference constructor compiled without FP
contraction. Rays are 8 float32 ``{pos, dir, tmin, tmax}`` (lbvh.h:388-401).

Generation order matters: the reference's leaf slot p holds primitive p in
input order, so tree quality follows input order. Each generator documents its
order.
"""
from __future__ import annotations

import math

import numpy as np



_C1, _C2, _C3 = np.uint64(0x9E3779B97F4A7C15), np.uint64(0xBF58476D1CE4E5B9), np.uint64(0x94D049BB133111EB)
_CHUNK = 1 << 16  # elements per block of the hash (a few L2-resident temporaries)


def _splitmix(x: np.ndarray, t: np.ndarray) -> None:
    """The splitmix64 finaliser applied to x in place (t: scratch)."""
    np.add(x, _C1, out=x)
    for shift, mul in ((30, _C2), (27, _C3)):
        np.right_shift(x, np.uint64(shift), out=t)
        np.bitwise_xor(x, t, out=x)
        np.multiply(x, mul, out=x)
    np.right_shift(x, np.uint64(31), out=t)
    np.bitwise_xor(x, t, out=x)


def uniform(seed: int, stream: int, n: int, start: int = 0) -> np.ndarray:
    """n float64 uniforms in [0, 1) (53-bit), element i keyed by start + i:
    splitmix64(splitmix64(i ^ key) + key) >> 11, scaled by 2^-53."""
    out = np.empty(n, np.float64)
    with np.errstate(over="ignore"):
        key = np.uint64((seed * 0x632BE59BD9B4E019 + stream * 0x85EBCA77C2B2AE63) & 0xFFFFFFFFFFFFFFFF)
        x, t = np.empty(_CHUNK, np.uint64), np.empty(_CHUNK, np.uint64)
        for a in range(0, n, _CHUNK):
            m = min(_CHUNK, n - a)
            xa, ta = x[:m], t[:m]
            xa[:] = np.arange(start + a, start + a + m, dtype=np.uint64)
            np.bitwise_xor(xa, key, out=xa)
            _splitmix(xa, ta)
            np.add(xa, key, out=xa)
            _splitmix(xa, ta)
            np.right_shift(xa, np.uint64(11), out=xa)
            np.multiply(xa, 1.0 / 9007199254740992.0, out=out[a : a + m], casting="unsafe")
    return out


def normal(seed: int, stream: int, n: int, start: int = 0) -> np.ndarray:
    """n standard normals by Box-Muller over two uniform streams."""
    u1 = uniform(seed, 2 * stream + 1000, n, start)
    u2 = uniform(seed, 2 * stream + 1001, n, start)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


def make_triangles(verts: np.ndarray) -> np.ndarray:
    """Reference ``triangle<float>(a, b, c)`` (lbvh.h:1967-1972) for n vertex
    triples ([n, 9] or [n, 3, 3]) -> [n, 12] float32. numpy float32 arithmetic
    rounds every product and difference, matching the reference built with
    -ffp-contract=off."""
    v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3, 3)
    a, b, c = v[:, 0], v[:, 1], v[:, 2]
    e0 = a - b
    e1 = c - a
    n = np.empty_like(e0)
    n[:, 0] = (e0[:, 1] * e1[:, 2]) - (e0[:, 2] * e1[:, 1])
    n[:, 1] = (e0[:, 2] * e1[:, 0]) - (e0[:, 0] * e1[:, 2])
    n[:, 2] = (e0[:, 0] * e1[:, 1]) - (e0[:, 1] * e1[:, 0])
    out = np.empty((v.shape[0], 12), np.float32)
    out[:, 0:3] = a
    out[:, 3:6] = e0
    out[:, 6:9] = e1
    out[:, 9:12] = n
    return out


def triangle_vertices(tris: np.ndarray) -> np.ndarray:
    """Inverse of make_triangles for the vertices: a = p0, b = p0 - e0,
    c = p0 + e1 (the reconstruction the reference converter uses)."""
    t = np.asarray(tris, dtype=np.float32).reshape(-1, 12)
    out = np.empty((t.shape[0], 3, 3), np.float32)
    out[:, 0] = t[:, 0:3]
    out[:, 1] = t[:, 0:3] - t[:, 3:6]
    out[:, 2] = t[:, 0:3] + t[:, 6:9]
    return out


# --------------------------------------------------------------------------
# scenes


def soup_vertices(n: int, seed: int, sigma: float = 0.03, start: int = 0) -> np.ndarray:
    """Random-order triangle soup: centroids uniform in [-1, 1]^3 and each
    vertex = centroid + N(0, sigma) per axis. Returns [n, 9] float32 vertices
    for triangles start .. start + n - 1."""
    c = uniform(seed, 0, 3 * n, 3 * start).reshape(n, 3) * 2.0 - 1.0
    off = normal(seed, 1, 9 * n, 9 * start).reshape(n, 3, 3) * sigma
    v = c[:, None, :] + off
    return v.reshape(n, 9).astype(np.float32)


def soup(n: int, seed: int, sigma: float = 0.03, chunk: int = 1 << 21) -> np.ndarray:
    """soup_vertices as reference triangles, generated in chunks (so 16M
    triangles need about 1 GB of temporaries, not 10)."""
    out = np.empty((n, 12), np.float32)
    for s in range(0, n, chunk):
        k = min(chunk, n - s)
        out[s : s + k] = make_triangles(soup_vertices(k, seed, sigma, start=s))
    return out


def soup_large(n: int, seed: int, sigma: float = 0.03, chunk: int = 1 << 22) -> np.ndarray:
    """The soup_vertices distribution for large n (the 16M-triangle build
    workload), drawn from numpy's PCG64 generator instead of the counter hash:
    about 10x faster, deterministic for a given seed and numpy version."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty((n, 12), np.float32)
    for s in range(0, n, chunk):
        k = min(chunk, n - s)
        c = rng.random((k, 1, 3), dtype=np.float32) * np.float32(2.0) - np.float32(1.0)
        v = c + rng.standard_normal((k, 3, 3), dtype=np.float32) * np.float32(sigma)
        out[s : s + k] = make_triangles(v)
    return out


def torus_scene(seed: int, major: float = 1.0, minor: float = 0.35,
                nu: int = 80, nv: int = 40, removed_quads: int = 40,
                plane_tris: int = 2000) -> np.ndarray:
    """Mid-size coherent scene: a parametric torus (axis along z, facing a
    camera on the +z axis) tessellated as nu x nv quads split into two
    triangles each, with `removed_quads` quads dropped by seed, followed by a
    ground plane of `plane_tris` triangles at y = -1.5.

    Defaults give 6,400 - 80 = 6,320 torus triangles plus 2,000 plane
    triangles. Order: torus in (u, v) grid order, then the plane row by row.
    """
    quads = nu * nv
    drop = np.argsort(uniform(seed, 10, quads), kind="stable")[:removed_quads]
    keep = np.ones(quads, bool)
    keep[drop] = False
    iu, iv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    iu = iu.reshape(-1)[keep]
    iv = iv.reshape(-1)[keep]

    def p(u, v):
        a = 2.0 * math.pi * u / nu
        b = 2.0 * math.pi * v / nv
        r = major + minor * np.cos(b)
        return np.stack([r * np.cos(a), r * np.sin(a), minor * np.sin(b)], -1)

    p00, p10 = p(iu, iv), p(iu + 1, iv)
    p01, p11 = p(iu, iv + 1), p(iu + 1, iv + 1)
    t1 = np.stack([p00, p10, p11], 1)
    t2 = np.stack([p00, p11, p01], 1)
    torus = np.stack([t1, t2], 1).reshape(-1, 3, 3)

    # ground plane: plane_tris / 2 quads on a near-square grid over [-4, 4]^2
    nq = plane_tris // 2
    gx = int(math.ceil(math.sqrt(nq)))
    gz = int(math.ceil(nq / gx))
    cells = np.arange(nq)
    cx, cz = cells % gx, cells // gx
    x0 = -4.0 + 8.0 * cx / gx
    x1 = -4.0 + 8.0 * (cx + 1) / gx
    z0 = -4.0 + 8.0 * cz / gz
    z1 = -4.0 + 8.0 * (cz + 1) / gz
    y = np.full(nq, -1.5)
    q00 = np.stack([x0, y, z0], -1)
    q10 = np.stack([x1, y, z0], -1)
    q01 = np.stack([x0, y, z1], -1)
    q11 = np.stack([x1, y, z1], -1)
    plane = np.stack([np.stack([q00, q01, q11], 1), np.stack([q00, q11, q10], 1)], 1).reshape(-1, 3, 3)
    return make_triangles(np.concatenate([torus, plane]).astype(np.float32))


def _quad_grid(o, du, dv, nu, nv):
    iu, iv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    iu = iu.reshape(-1)
    iv = iv.reshape(-1)
    def p(a, b):
        return o[None] + (a / nu)[:, None] * du[None] + (b / nv)[:, None] * dv[None]
    p00, p10, p01, p11 = p(iu, iv), p(iu + 1, iv), p(iu, iv + 1), p(iu + 1, iv + 1)
    return np.stack([np.stack([p00, p10, p11], 1), np.stack([p00, p11, p01], 1)], 1).reshape(-1, 3, 3)


def room_scene(seed: int, n: int = 262_267) -> np.ndarray:
    """Large clustered scene in a room of [-10, 10] x [0, 6] x [-10, 10]:
    about 10% axis-aligned wall/floor/ceiling quads subdivided into triangle
    pairs, 60% in 64 cylindrical columns (radius 0.05-0.2, floor to ceiling),
    and the rest small clutter triangles clustered N(0, 0.05) around 500
    seeded centres with log-normal(sigma = 1.5) areas. Exactly n triangles.
    Order: each wall, then each column, then each cluster, contiguously."""
    n_wall = int(round(0.10 * n))
    n_col = int(round(0.60 * n))
    n_clut = n - n_wall - n_col
    lo, hi = np.array([-10.0, 0.0, -10.0]), np.array([10.0, 6.0, 10.0])
    X, Y, Z = np.eye(3)
    size = hi - lo
    faces = [  # origin, du, dv
        (lo, X * size[0], Z * size[2]),                        # floor
        (np.array([lo[0], hi[1], lo[2]]), Z * size[2], X * size[0]),  # ceiling
        (lo, Y * size[1], X * size[0]),                        # wall z = lo
        (np.array([lo[0], lo[1], hi[2]]), X * size[0], Y * size[1]),  # wall z = hi
        (lo, Z * size[2], Y * size[1]),                        # wall x = lo
        (np.array([hi[0], lo[1], lo[2]]), Y * size[1], Z * size[2]),  # wall x = hi
    ]
    per_face = -(-n_wall // 6)
    walls = []
    for o, du, dv in faces:
        q = -(-per_face // 2)
        nu = max(1, int(math.sqrt(q)))
        nv = -(-q // nu)
        walls.append(_quad_grid(o, du, dv, nu, nv))
    walls = np.concatenate(walls)[:n_wall]

    # columns
    ncols = 64
    cpos = uniform(seed, 20, 2 * ncols).reshape(ncols, 2) * 18.0 - 9.0
    crad = 0.05 + 0.15 * uniform(seed, 21, ncols)
    per_col = np.full(ncols, n_col // ncols)
    per_col[: n_col % ncols] += 1
    cols = []
    for k in range(ncols):
        m = int(per_col[k])
        q = -(-m // 2)
        seg = 24
        rings = -(-q // seg)
        iu, iv = np.meshgrid(np.arange(seg), np.arange(rings), indexing="ij")
        iu = iu.reshape(-1)
        iv = iv.reshape(-1)
        def p(a, b, k=k, rings=rings):
            ang = 2.0 * math.pi * a / seg
            return np.stack([cpos[k, 0] + crad[k] * np.cos(ang),
                             lo[1] + size[1] * b / rings,
                             cpos[k, 1] + crad[k] * np.sin(ang)], -1)
        p00, p10, p01, p11 = p(iu, iv), p(iu + 1, iv), p(iu, iv + 1), p(iu + 1, iv + 1)
        t = np.stack([np.stack([p00, p10, p11], 1), np.stack([p00, p11, p01], 1)], 1).reshape(-1, 3, 3)
        cols.append(t[:m])
    cols = np.concatenate(cols)

    # clutter around 500 centres on/above the floor
    ncl = 500
    cc = np.stack([uniform(seed, 30, ncl) * 18.0 - 9.0,
                   0.2 + uniform(seed, 31, ncl) * 2.5,
                   uniform(seed, 32, ncl) * 18.0 - 9.0], -1)
    owner = np.minimum((uniform(seed, 33, n_clut) * ncl).astype(np.int64), ncl - 1)
    owner = np.sort(owner, kind="stable")  # contiguous clusters
    cen = cc[owner] + normal(seed, 34, 3 * n_clut).reshape(-1, 3) * 0.05
    area = np.exp(math.log(2e-4) + 1.5 * normal(seed, 35, n_clut))
    edge = np.sqrt(4.0 * area / math.sqrt(3.0))
    d = normal(seed, 36, 9 * n_clut).reshape(-1, 3, 3)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    clut = cen[:, None, :] + d * (edge[:, None, None] / math.sqrt(3.0))
    allv = np.concatenate([walls, cols, clut]).astype(np.float32)
    assert allv.shape[0] == n
    return make_triangles(allv)


# --------------------------------------------------------------------------
# rays


def _rays(pos: np.ndarray, d: np.ndarray, tmin: float = 0.0, tmax: float = math.inf) -> np.ndarray:
    out = np.empty((d.shape[0], 8), np.float32)
    out[:, 0:3] = pos
    out[:, 3:6] = d
    out[:, 6] = tmin
    out[:, 7] = tmax
    return out


def pinhole_rays(width: int, height: int, eye=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0),
                 up=(0.0, 1.0, 0.0), fov_deg: float = 60.0) -> np.ndarray:
    """Primary rays, row-major from the top-left pixel, through pixel centres
    of a pinhole camera with a vertical field of view of fov_deg. Directions
    are unit length; tmin = 0, tmax = +inf."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    th = math.tan(math.radians(fov_deg) / 2.0)
    asp = width / height
    ys, xs = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    xn = ((xs.reshape(-1) + 0.5) / width * 2.0 - 1.0) * th * asp
    yn = (1.0 - (ys.reshape(-1) + 0.5) / height * 2.0) * th
    d = f[None] + xn[:, None] * r[None] + yn[:, None] * u[None]
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    return _rays(np.broadcast_to(eye, d.shape), d)


def sphere_dirs(seed: int, stream: int, m: int) -> np.ndarray:
    z = uniform(seed, stream, m) * 2.0 - 1.0
    phi = uniform(seed, stream + 1, m) * 2.0 * math.pi
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], -1)


def scene_box(tris: np.ndarray):
    v = triangle_vertices(tris).reshape(-1, 3).astype(np.float64)
    return v.min(0), v.max(0)


def incoherent_rays(tris: np.ndarray, m: int, seed: int, scale: float = 1.5) -> np.ndarray:
    """m rays with origins uniform in the scene box scaled by `scale` about
    its centre and directions uniform on the unit sphere."""
    lo, hi = scene_box(tris)
    c = 0.5 * (lo + hi)
    h = 0.5 * (hi - lo) * scale
    o = c + (uniform(seed, 40, 3 * m).reshape(m, 3) * 2.0 - 1.0) * h
    return _rays(o, sphere_dirs(seed, 41, m))


def diffuse_bounce(rays: np.ndarray, hits: np.ndarray, tris: np.ndarray, seed: int,
                   eps: float = 1e-4) -> np.ndarray:
    """One cosine-weighted diffuse bounce per hit: origin at the hit point
    (pos + t * dir) pushed eps along the geometric normal facing the incoming
    ray, direction cosine-distributed about that normal, random numbers keyed
    by the ray index. Returns bounce rays for the hit rays only, in ray
    order (misses are skipped)."""
    prim = hits["prim"]
    sel = np.nonzero(prim != 0xFFFFFFFF)[0]
    r = np.asarray(rays, np.float64)[sel]
    t = hits["t"][sel].astype(np.float64)
    nrm = np.asarray(tris, np.float64)[prim[sel], 9:12]
    nrm /= np.maximum(np.linalg.norm(nrm, axis=-1, keepdims=True), 1e-30)
    flip = np.sum(nrm * r[:, 3:6], -1) > 0
    nrm[flip] = -nrm[flip]
    p = r[:, 0:3] + t[:, None] * r[:, 3:6] + eps * nrm
    # keyed by the index of the incoming ray
    top = int(sel.max()) + 1 if sel.size else 0
    u1 = uniform(seed, 50, top)[sel]
    u2 = uniform(seed, 51, top)[sel]
    rr = np.sqrt(u1)
    phi = 2.0 * math.pi * u2
    lx, ly, lz = rr * np.cos(phi), rr * np.sin(phi), np.sqrt(np.maximum(0.0, 1.0 - u1))
    a = np.where(np.abs(nrm[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    tx = np.cross(a, nrm)
    tx /= np.linalg.norm(tx, axis=-1, keepdims=True)
    ty = np.cross(nrm, tx)
    d = lx[:, None] * tx + ly[:, None] * ty + lz[:, None] * nrm
    return _rays(p, d)


def log_uniform_counts(k: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """k integers log-uniform in [lo, hi]."""
    u = uniform(seed, 60, k)
    return np.minimum(hi, np.floor(np.exp(math.log(lo) + u * (math.log(hi + 1) - math.log(lo))))).astype(np.int64)


def random_rays_in_box(lo, hi, m: int, seed: int, stream: int = 70, scale: float = 1.5) -> np.ndarray:
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    h = 0.5 * (hi - lo) * scale
    o = c + (uniform(seed, stream, 3 * m).reshape(m, 3) * 2.0 - 1.0) * h
    return _rays(o, sphere_dirs(seed, stream + 1, m))


def batch_scene(k: int = 4096, lo: int = 64, hi: int = 65536, rays_per_mesh: int = 4096, seed: int = 3):
    """Batched workload: k independent random-order soups (each as
    soup_vertices, centroids uniform in [-1, 1]^3, drawn with its own seed
    base + i) with triangle counts log-uniform in [lo, hi], concatenated,
    and rays_per_mesh random rays per mesh (origins uniform in the 1.5x box of
    the soups' common extent, directions uniform on the sphere).
    Returns (triangles [total, 12], offsets [k + 1] uint32, rays, ray_offsets)."""
    counts = log_uniform_counts(k, lo, hi, seed)
    offsets = np.zeros(k + 1, np.uint32)
    offsets[1:] = np.cumsum(counts)
    tris = np.empty((int(offsets[-1]), 12), np.float32)
    for i in range(k):
        tris[offsets[i] : offsets[i + 1]] = soup_large(int(counts[i]), seed * 1_000_003 + i)
    rays = random_rays_in_box([-1.0] * 3, [1.0] * 3, k * rays_per_mesh, seed, stream=80)
    ray_offsets = (np.arange(k + 1, dtype=np.int64) * rays_per_mesh).astype(np.uint32)
    return tris, offsets, rays, ray_offsets


def torus_mesh(n_target: int, seed: int, major: float = 1.0, minor: float = 0.35) -> np.ndarray:
    """A torus tessellated to about n_target triangles in (u, v) grid order
    (coherent input order, so the reference's leaf order gives a usable tree),
    placed at a seeded offset."""
    quads = max(1, n_target // 2)
    nv = max(3, int(round(math.sqrt(quads / 2.0))))
    nu = max(3, quads // nv)
    iu, iv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    iu = iu.reshape(-1)
    iv = iv.reshape(-1)
    shift = (uniform(seed, 90, 3) * 2.0 - 1.0) * 2.0

    def p(u, v):
        a = 2.0 * math.pi * u / nu
        b = 2.0 * math.pi * v / nv
        r = major + minor * np.cos(b)
        return np.stack([r * np.cos(a), r * np.sin(a), minor * np.sin(b)], -1) + shift

    p00, p10 = p(iu, iv), p(iu + 1, iv)
    p01, p11 = p(iu, iv + 1), p(iu + 1, iv + 1)
    t = np.stack([np.stack([p00, p10, p11], 1), np.stack([p00, p11, p01], 1)], 1).reshape(-1, 3, 3)
    return make_triangles(t.astype(np.float32))


def jitter(tris: np.ndarray, seed: int, sigma: float = 0.01) -> np.ndarray:
    """Seeded vertex jitter N(0, sigma) of every triangle's vertices (the
    served workload's refit input)."""
    v = triangle_vertices(tris).reshape(-1, 9).astype(np.float64)
    v += normal(seed, 95, v.size).reshape(v.shape) * sigma
    return make_triangles(v.astype(np.float32))


def served_requests(n_requests: int, rate: float, seed: int, n_scenes: int = 48, lo: int = 1000, hi: int = 2_000_000,
                    ray_lo: int = 16384, ray_hi: int = 2_000_000, ray_pool: int = 4):
    """Served workload: Poisson arrivals at `rate` requests/s. First one build
    per scene (sizes log-uniform in [lo, hi] triangles, torus meshes), then a
    seeded mix of 70% traces (log-uniform [ray_lo, ray_hi] rays, a slice of a
    pooled incoherent ray set), 20% refits (vertex jitter N(0, 0.01); each
    scene alternates between two jittered variants of its mesh) and 10% full
    rebuilds (of the scene's unjittered mesh), each on a uniformly chosen
    scene. Returns [(arrival_s, kind, scene, data)] in arrival order; data
    arrays are shared between requests."""
    sizes = log_uniform_counts(n_scenes, lo, hi, seed)
    meshes = [torus_mesh(int(sizes[s]), seed * 7919 + s) for s in range(n_scenes)]
    variants = [(jitter(m, seed * 31 + 2 * s), jitter(m, seed * 31 + 2 * s + 1)) for s, m in enumerate(meshes)]
    pool = [incoherent_rays(meshes[k % n_scenes], ray_hi, seed + 100 + k, scale=1.2) for k in range(ray_pool)]
    gaps = -np.log1p(-uniform(seed, 96, n_requests)) / rate
    t = np.cumsum(gaps)
    kinds = uniform(seed, 97, n_requests)
    who = np.minimum((uniform(seed, 98, n_requests) * n_scenes).astype(np.int64), n_scenes - 1)
    nr = log_uniform_counts(n_requests, ray_lo, ray_hi, seed + 1)
    flip = [0] * n_scenes
    out = []
    for i in range(n_requests):
        if i < n_scenes:
            out.append((float(t[i]), "build", i, meshes[i]))
            continue
        s = int(who[i])
        if kinds[i] < 0.7:
            rays = pool[i % ray_pool]
            start = int(uniform(seed, 99, 1, i)[0] * (rays.shape[0] - nr[i]))
            out.append((float(t[i]), "trace", s, rays[start : start + int(nr[i])]))
        elif kinds[i] < 0.9:
            out.append((float(t[i]), "refit", s, variants[s][flip[s]]))
            flip[s] ^= 1
        else:
            out.append((float(t[i]), "build", s, meshes[s]))
    return out


def example_spheres() -> np.ndarray:
    """The three spheres of the reference's example program
    (examples/minimal.cpp:48-50), as {radius, x, y, z} rows."""
    return np.array([[1, 5, 1, -5], [1, 0, 2, -5], [1, -5, 1, -5]], np.float32)


def example_camera_rays(width: int, height: int) -> np.ndarray:
    """The example program's camera (examples/minimal.cpp:140-160) at a
    chosen resolution: origin (0, 0, 5), direction {x_ndc * aspect * 0.75,
    y_ndc * 0.75, -1} through pixel centres, row-major from the top; tmin = 0,
    tmax = +inf. Computed in float32."""
    f32 = np.float32
    x = (np.arange(width, dtype=f32) + f32(0.5))
    y = (np.arange(height, dtype=f32) + f32(0.5))
    x_ndc = (f32(2) * x / f32(width)) - f32(1)
    y_ndc = -(f32(2) * y / f32(height)) + f32(1)
    aspect = f32(width) / f32(height)
    fov = f32(0.75)
    out = np.zeros((height, width, 8), f32)
    out[..., 2] = 5
    out[..., 3] = (x_ndc * aspect * fov)[None, :]
    out[..., 4] = (y_ndc * fov)[:, None]
    out[..., 5] = -1
    out[..., 7] = np.inf
    return out.reshape(-1, 8)


def sphere_scene(n: int, seed: int, extent: float = 6.0, r_lo: float = 0.02, r_hi: float = 0.3) -> np.ndarray:
    """n spheres {radius, x, y, z}: centres uniform in a cube of side
    `extent` about the origin, radii uniform in [r_lo, r_hi]."""
    u = uniform(seed, 80, 4 * n).reshape(n, 4)
    out = np.empty((n, 4), np.float32)
    out[:, 0] = r_lo + (r_hi - r_lo) * u[:, 0]
    out[:, 1:] = (u[:, 1:] - 0.5) * extent
    return out
