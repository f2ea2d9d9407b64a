"""Python host interface over the C ABI, mirroring the reference's API.

Reference (tay10r/lbvh, lbvh.h)            here
-----------------------------------------  -----------------------------------
triangle<float>(a, b, c)  (1967-1972)      make_triangles(verts)  (GPU kernel)
builder<float>            (312-353)        Builder
  operator()(prims, count, converter)      Builder.__call__(prims, count, converter)
  triangle_aabb_converter<float> (1988)    TRIANGLES (default converter)
  user aabb_converter functor (342-345)    any callable, or BOXES for ready boxes
bvh<float>                (259-299)        BVH (size(), at(i), [i], nodes())
traverser<float, P, I>    (502-534)        Traverser
  operator()(ray, triangle_intersector)    Traverser.__call__(rays)
intersection_container    (359-382)        HIT_DTYPE records {prim, t, u, v}

Arrays may be numpy arrays (host) or torch tensors (host or CUDA); the
library detects where each one lives. Results for host inputs come back as
numpy arrays; for CUDA inputs they are written to CUDA tensors.

Error behaviour: the reference has none (everything is noexcept and n < 2 is
undefined behaviour, lbvh.h:1812, 1835-1838). Here invalid input raises
ValueError before any work, and device failures raise LbvhError.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import LbvhError

NODE_DTYPE = np.dtype(
    [("lo", "<f4", (3,)), ("hi", "<f4", (3,)), ("left", "<u4"), ("right", "<u4")]
)
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
# lbvh_sphere_hit: the example program's sphere_hit {tmin, uv, normal} with
# the hit sphere's index (examples/minimal.cpp:24-42)
SPHERE_HIT_DTYPE = np.dtype(
    [("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("normal", "<f4", (3,)), ("pad", "<f4")]
)
LEAF_BIT = _lib.LEAF_BIT
MISS = _lib.MISS

TRIANGLES = "triangles"  # triangle_aabb_converter<float>
BOXES = "boxes"          # primitives are already boxes (identity converter)

try:  # torch is plumbing (device memory, streams), not required for host use
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_tensor(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


def _addr(x) -> int:
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return x.ctypes.data
    if _is_tensor(x):
        if not x.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return x.data_ptr()
    raise TypeError(f"expected a numpy array or torch tensor, got {type(x).__name__}")


def _rows(x, width: int, name: str) -> int:
    if isinstance(x, np.ndarray):
        if x.dtype != np.float32:
            raise ValueError(f"{name} must be float32")
        size = x.size
    elif _is_tensor(x):
        if x.dtype != torch.float32:
            raise ValueError(f"{name} must be float32")
        size = x.numel()
    else:
        raise TypeError(f"{name}: expected a numpy array or torch tensor")
    if size % width:
        raise ValueError(f"{name}: {size} floats is not a multiple of {width}")
    return size // width


def _is_cuda(x) -> bool:
    return _is_tensor(x) and x.is_cuda


class Context:
    """A device + stream + workspace (lbvh_ctx). One per host thread."""

    def __init__(self, device: int | None = None, stream: int | None = None):
        L = _lib.lib()
        if device is None:
            device = torch.cuda.current_device() if (torch is not None and torch.cuda.is_available()) else 0
        if stream is None and torch is not None and torch.cuda.is_available():
            stream = torch.cuda.current_stream(device).cuda_stream
        self.device = device
        self.stream = stream or 0
        h = ctypes.c_void_p()
        st = L.lbvh_ctx_create(device, ctypes.c_void_p(self.stream), ctypes.byref(h))
        if st != 0:
            raise LbvhError(st, f"context creation failed: {_lib.status_string(st)}")
        self._h = h

    @property
    def handle(self):
        return self._h

    def check(self, st: int):
        if st != 0:
            msg = _lib.lib().lbvh_ctx_last_error(self._h).decode()
            if st == _lib.LBVH_ERR_INVALID_ARG:
                raise ValueError(msg)
            raise LbvhError(st, msg)

    def synchronize(self):
        self.check(_lib.lib().lbvh_ctx_synchronize(self._h))

    def set_param(self, param: int, value: int):
        self.check(_lib.lib().lbvh_ctx_set_param(self._h, param, value))

    def reserve(self, n_prims: int, n_rays: int = 0):
        self.check(_lib.lib().lbvh_ctx_reserve(self._h, n_prims, n_rays))

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().lbvh_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default: dict[int, Context] = {}


def default_context() -> Context:
    dev = torch.cuda.current_device() if (torch is not None and torch.cuda.is_available()) else 0
    if dev not in _default:
        _default[dev] = Context(dev)
    return _default[dev]


def make_triangles(verts, out=None, ctx: Context | None = None):
    """Reference triangle<float>(a, b, c) for n vertex triples, on the GPU.
    verts: [n, 9] float32 -> [n, 12] float32 (numpy for host input)."""
    ctx = ctx or default_context()
    n = _rows(verts, 9, "verts")
    if out is None:
        if _is_cuda(verts):
            out = torch.empty((n, 12), dtype=torch.float32, device=verts.device)
        else:
            out = np.empty((n, 12), np.float32)
    ctx.check(_lib.lib().lbvh_make_triangles(ctx.handle, _addr(verts), n, _addr(out)))
    return out


class BVH:
    """A device-resident BVH (lbvh::bvh<float>): n - 1 internal nodes of 32
    bytes, nodes[0] the root, leaf references flagged by LEAF_BIT."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        self.ctx.check(_lib.lib().lbvh_bvh_create(self.ctx.handle, ctypes.byref(h)))
        self._h = h
        self._keep = None  # keeps borrowed device primitives alive
        self._host_nodes = None
        self.kind = None

    @property
    def handle(self):
        return self._h

    def info(self):
        n = ctypes.c_size_t()
        nn = ctypes.c_size_t()
        fl = ctypes.c_uint32()
        _lib.lib().lbvh_bvh_info(self._h, ctypes.byref(n), ctypes.byref(nn), ctypes.byref(fl))
        return n.value, nn.value, fl.value

    @property
    def num_primitives(self) -> int:
        return self.info()[0]

    def size(self) -> int:
        """bvh<float>::size(): the number of internal nodes."""
        return self.info()[1]

    __len__ = size

    def nodes(self, out=None):
        """All nodes: a NODE_DTYPE numpy array, or written into `out` (a
        numpy array or CUDA tensor of (n - 1) * 32 bytes)."""
        if out is None:
            out = np.empty(self.size(), NODE_DTYPE)
        self.ctx.check(_lib.lib().lbvh_bvh_nodes(self.ctx.handle, self._h, _addr(out)))
        return out

    def device_nodes_ptr(self) -> int:
        return _lib.lib().lbvh_bvh_device_nodes(self._h) or 0

    def at(self, i: int):
        """bvh<float>::at(): bounds-checked node access (IndexError)."""
        if not 0 <= i < self.size():
            raise IndexError(i)
        return self[i]

    def __getitem__(self, i):
        if self._host_nodes is None:
            self._host_nodes = self.nodes()
        return self._host_nodes[i]

    def curve(self):
        """(codes, sorted_codes, stable_perm, centroid_bounds[6]) of a build
        made with keep_curve=True."""
        n = self.num_primitives
        codes = np.empty(n, np.uint32)
        sc = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        bounds = np.empty(6, np.float32)
        self.ctx.check(_lib.lib().lbvh_bvh_curve(self.ctx.handle, self._h, _addr(codes), _addr(sc),
                                                 _addr(perm), _addr(bounds)))
        return codes, sc, perm, bounds

    @classmethod
    def from_nodes(cls, nodes, triangles, ctx: Context | None = None) -> "BVH":
        """A BVH over an existing node array (NODE_DTYPE records, e.g. one
        made by the reference's builder) and its n_nodes + 1 triangles, for
        tracing. The array is checked on the device (LbvhError on a node
        array that is not a tree over its leaves)."""
        bvh = cls(ctx)
        if isinstance(nodes, np.ndarray):
            nodes = np.ascontiguousarray(nodes)
            n_nodes = nodes.nbytes // 32
        else:
            n_nodes = nodes.numel() * nodes.element_size() // 32
        if _rows(triangles, 12, "triangles") != n_nodes + 1:
            raise ValueError("need n_nodes + 1 triangles")
        bvh.ctx.check(_lib.lib().lbvh_bvh_import_triangles(bvh.ctx.handle, _addr(nodes), n_nodes,
                                                          _addr(triangles), bvh.handle))
        bvh.kind = TRIANGLES
        bvh._keep = triangles if _is_cuda(triangles) else None
        return bvh

    def primitives(self, out=None):
        """The primitives the BVH reads, in input order: [n, 12] float32
        triangles or [n, 6] boxes (numpy, or written into `out`)."""
        n, _, _ = self.info()
        if out is None:
            out = np.empty((n, 12 if self.kind == TRIANGLES else 6), np.float32)
        self.ctx.check(_lib.lib().lbvh_bvh_primitives(self.ctx.handle, self._h, _addr(out)))
        return out

    # -- raw dump / reload ----------------------------------------------------
    _MAGIC = "lbvh_gb300.bvh"
    _VERSION = 1

    def save(self, path) -> None:
        """Writes the raw dump of a triangle BVH built in reference leaf
        order: the node array (the reference's 32-byte nodes) and the
        triangles, as an .npz file. BVH.load reads it back."""
        n, _, flags = self.info()
        if self.kind != TRIANGLES or flags & _lib.LBVH_BUILD_SORTED_LEAVES:
            raise ValueError("save() writes triangle BVHs in reference leaf order")
        np.savez(path, magic=np.array(self._MAGIC), version=np.array(self._VERSION, np.int32),
                 nodes=self.nodes().view(np.uint8).reshape(-1, 32), triangles=self.primitives())

    @classmethod
    def load(cls, path, ctx: Context | None = None) -> "BVH":
        """Reads a dump written by save(); the node array is checked on the
        device before the BVH can be traced (from_nodes)."""
        with np.load(path) as f:
            if str(f["magic"]) != cls._MAGIC or int(f["version"]) != cls._VERSION:
                raise ValueError(f"{path} is not a BVH dump of this library (version {cls._VERSION})")
            nodes = np.ascontiguousarray(f["nodes"]).reshape(-1).view(NODE_DTYPE)
            tris = np.ascontiguousarray(f["triangles"], dtype=np.float32)
        return cls.from_nodes(nodes, tris, ctx)

    def refit(self, primitives):
        """Recompute all node boxes over moved primitives (same count and
        order as the build input), keeping the topology."""
        n = self.num_primitives
        L = _lib.lib()
        self._host_nodes = None
        if self.kind == TRIANGLES:
            if _rows(primitives, 12, "triangles") != n:
                raise ValueError("refit needs the build's primitive count")
            self.ctx.check(L.lbvh_refit_triangles(self.ctx.handle, self._h, _addr(primitives)))
        else:
            if _rows(primitives, 6, "boxes") != n:
                raise ValueError("refit needs the build's primitive count")
            self.ctx.check(L.lbvh_refit_boxes(self.ctx.handle, self._h, _addr(primitives)))
        if _is_cuda(primitives):
            self._keep = primitives
        return self

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().lbvh_bvh_destroy(self.ctx.handle, self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Builder:
    """lbvh::builder<float> on the GPU.

    Builder()(triangles)                      reference parity (default)
    Builder(sorted_leaves=True)(triangles)    intended LBVH: leaves in Morton order
    Builder()(boxes, converter=BOXES)         caller-converted boxes
    Builder()(objects, converter=fn)          fn(objects) -> [n, 6] boxes on the host
    """

    def __init__(self, ctx: Context | None = None, sorted_leaves: bool = False, keep_curve: bool = False):
        self.ctx = ctx or default_context()
        self.flags = (_lib.LBVH_BUILD_SORTED_LEAVES if sorted_leaves else 0) | (
            _lib.LBVH_BUILD_KEEP_CURVE if keep_curve else 0)

    def __call__(self, primitives, count: int | None = None, converter=TRIANGLES, into: BVH | None = None) -> BVH:
        bvh = into if into is not None else BVH(self.ctx)
        bvh._host_nodes = None
        L = _lib.lib()
        if callable(converter):
            boxes = np.ascontiguousarray(converter(primitives), dtype=np.float32).reshape(-1, 6)
            primitives, converter = boxes, BOXES
        if converter == TRIANGLES:
            n = _rows(primitives, 12, "triangles")
            fn = L.lbvh_build_triangles
        elif converter == BOXES:
            n = _rows(primitives, 6, "boxes")
            fn = L.lbvh_build_boxes
        else:
            raise ValueError(f"unknown converter {converter!r}")
        if count is not None:
            if count > n:
                raise ValueError("count exceeds the primitive array")
            n = count
        if n < 2:
            raise ValueError(f"a BVH needs at least 2 primitives (got {n})")
        self.ctx.check(fn(self.ctx.handle, _addr(primitives), n, self.flags, bvh.handle))
        bvh.kind = converter
        bvh._keep = primitives if _is_cuda(primitives) else None
        return bvh


class Traverser:
    """lbvh::traverser<float, triangle<float>, triangle_intersection<float>>
    with triangle_intersector<float>: closest hit per ray, bit-identical to
    the reference. The primitives are the ones the BVH was built over."""

    def __init__(self, bvh: BVH):
        if bvh.kind != TRIANGLES:
            raise ValueError("the built-in traverser intersects triangles")
        self.bvh = bvh
        self.ctx = bvh.ctx

    def __call__(self, rays, out=None, counts: bool = False):
        """rays: [m, 8] float32 {pos, dir, tmin, tmax} (or one ray of 8).
        Returns HIT_DTYPE records (numpy for host rays; for CUDA rays a
        [m, 4] tensor whose rows view as {prim, t, u, v}). With counts=True
        also returns per-ray box-test and triangle-test counts."""
        m = _rows(rays, 8, "rays")
        cuda = _is_cuda(rays)
        if out is None:
            if cuda:
                out = torch.empty((m, 4), dtype=torch.float32, device=rays.device)
            else:
                out = np.empty(m, HIT_DTYPE)
        L = _lib.lib()
        if counts:
            if cuda:
                nb = torch.empty(m, dtype=torch.int32, device=rays.device)
                nt = torch.empty(m, dtype=torch.int32, device=rays.device)
            else:
                nb = np.empty(m, np.uint32)
                nt = np.empty(m, np.uint32)
            self.ctx.check(L.lbvh_trace_triangles_counts(self.ctx.handle, self.bvh.handle, _addr(rays), m,
                                                         _addr(out), _addr(nb), _addr(nt)))
            return out, nb, nt
        self.ctx.check(L.lbvh_trace_triangles(self.ctx.handle, self.bvh.handle, _addr(rays), m, _addr(out)))
        return out


def sphere_boxes(spheres) -> np.ndarray:
    """The example program's sphere_to_box converter (examples/minimal.cpp:
    62-67) for {radius, x, y, z} rows: {pos - radius, pos + radius}, float32.
    It runs on the host, as the reference runs a caller's converter; build
    with Builder()(boxes, converter=BOXES)."""
    s = np.ascontiguousarray(spheres, dtype=np.float32).reshape(-1, 4)
    r = s[:, :1]
    return np.ascontiguousarray(np.concatenate([s[:, 1:] - r, s[:, 1:] + r], axis=1), dtype=np.float32)


class SphereTraverser:
    """traverser<float, sphere, sphere_hit> with the example program's
    intersector, run on the device (lbvh_trace_spheres): the user-primitive
    path. `bvh` is built from sphere_boxes(spheres) in reference leaf order;
    hit index, t and normal are bit-identical to the reference, u and v agree
    to within a few units in the last place (atan2 / acos)."""

    def __init__(self, bvh: BVH, spheres):
        if bvh.info()[2] & _lib.LBVH_BUILD_SORTED_LEAVES:
            raise ValueError("sphere traces need a BVH in reference leaf order")
        self.bvh = bvh
        self.ctx = bvh.ctx
        self.spheres = spheres if _is_cuda(spheres) else np.ascontiguousarray(spheres, dtype=np.float32)
        if _rows(self.spheres, 4, "spheres") != len(bvh) + 1:
            raise ValueError("need one sphere per leaf")

    def __call__(self, rays, out=None):
        m = _rows(rays, 8, "rays")
        if out is None:
            if _is_cuda(rays):
                out = torch.empty((m, 8), dtype=torch.float32, device=rays.device)
            else:
                out = np.empty(m, SPHERE_HIT_DTYPE)
        self.ctx.check(_lib.lib().lbvh_trace_spheres(self.ctx.handle, self.bvh.handle, _addr(self.spheres),
                                                     _addr(rays), m, _addr(out)))
        return out


def hits_view(t) -> np.ndarray:
    """HIT_DTYPE view of a [m, 4] float32 hits tensor copied to the host."""
    a = t.detach().cpu().numpy() if _is_tensor(t) else np.asarray(t)
    return np.ascontiguousarray(a).view(HIT_DTYPE).reshape(-1)


def _u32(x, name):
    if isinstance(x, np.ndarray):
        if x.dtype != np.uint32:
            raise ValueError(f"{name} must be uint32")
        return x
    if _is_tensor(x):
        if x.dtype not in (torch.int32, getattr(torch, "uint32", torch.int32)):
            raise ValueError(f"{name} must be a 32-bit integer tensor")
        return x
    return np.ascontiguousarray(x, dtype=np.uint32)


class Batch:
    """Many independent meshes built and traced together (one persistent
    launch each). Mesh k is triangles [offsets[k], offsets[k + 1]) of one
    concatenated [total, 12] array; the result per mesh equals the reference
    builder / traverser run on that mesh alone (mesh-local node and primitive
    indices)."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        self.ctx.check(_lib.lib().lbvh_batch_create(self.ctx.handle, ctypes.byref(h)))
        self._h = h
        self._keep = None
        self._offsets = None
        self._offsets_host = None

    def build(self, triangles, offsets, sorted_leaves: bool = False) -> "Batch":
        """Builds every mesh [offsets[k], offsets[k + 1]) in one launch; with
        sorted_leaves=True each mesh's tree is the sorted-leaf build of that
        mesh (leaves in stable Morton order; hits report input-order ids)."""
        offsets = _u32(offsets, "offsets")
        n_meshes = (offsets.size if isinstance(offsets, np.ndarray) else offsets.numel()) - 1
        total = _rows(triangles, 12, "triangles")
        if n_meshes < 1:
            raise ValueError("need at least one mesh")
        flags = _lib.LBVH_BUILD_SORTED_LEAVES if sorted_leaves else 0
        self.ctx.check(_lib.lib().lbvh_batch_build(self.ctx.handle, _addr(triangles), total, _addr(offsets),
                                                  n_meshes, flags, self._h))
        self._keep = (triangles, offsets)
        self._offsets = offsets  # read back lazily: build() stays free of host syncs
        self._offsets_host = None
        return self

    @property
    def offsets(self) -> np.ndarray:
        if self._offsets_host is None and self._offsets is not None:
            o = self._offsets
            self._offsets_host = o if isinstance(o, np.ndarray) else o.cpu().numpy().view(np.uint32)
        return self._offsets_host

    def info(self):
        a, b, c = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _lib.lib().lbvh_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def nodes(self, out=None):
        """All node blocks (NODE_DTYPE); mesh k's block starts at offsets[k] - k."""
        if out is None:
            out = np.empty(self.info()[2], NODE_DTYPE)
        self.ctx.check(_lib.lib().lbvh_batch_nodes(self.ctx.handle, self._h, _addr(out)))
        return out

    def mesh_nodes(self, k: int, all_nodes=None):
        nodes = self.nodes() if all_nodes is None else all_nodes
        o = self.offsets
        start = int(o[k]) - k
        return nodes[start : start + int(o[k + 1] - o[k]) - 1]

    def trace(self, rays, ray_offsets, out=None):
        """rays [m, 8]; rays [ray_offsets[k], ray_offsets[k + 1]) hit mesh k."""
        ray_offsets = _u32(ray_offsets, "ray_offsets")
        m = _rows(rays, 8, "rays")
        if out is None:
            if _is_cuda(rays):
                out = torch.empty((m, 4), dtype=torch.float32, device=rays.device)
            else:
                out = np.empty(m, HIT_DTYPE)
        self.ctx.check(_lib.lib().lbvh_batch_trace_triangles(self.ctx.handle, self._h, _addr(rays),
                                                            _addr(ray_offsets), m, _addr(out)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().lbvh_batch_destroy(self.ctx.handle, self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
