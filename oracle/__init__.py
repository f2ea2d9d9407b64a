"""ORACLE -- test infrastructure, not product code.

ctypes access to two CPU implementations of the reference LBVH path
(tay10r/lbvh, header ``lbvh.h``):

* ``port``: ``liboracle.so``, our C++ restatement (``lbvh_oracle.cpp``). It is
  built on every machine, including the GPU host.
* ``ref``: ``_ref/libref.so``, the unmodified reference header compiled through
  ``ref_shim.cpp``. It exists where the reference's files were present at
  build time (a reference checkout, or the copy ``stage_ref.sh`` puts in
  ``baseline/_ref``, which travels with the working tree), and is used to pin
  ``port``, to make golden fixtures and as the timed CPU baseline.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
use this package, and only as the checker or as the timed CPU baseline.

Array conventions (all little-endian, C-contiguous):
  triangles  float32 [n, 12]  {p0, e0, e1, normal}  (lbvh.h:1959-1983)
  boxes      float32 [n, 6]   {min, max}            (lbvh.h:208-215)
  nodes      void    [n-1]    32-byte records, see NODE_DTYPE (lbvh.h:220-255)
  rays       float32 [m, 8]   {pos, dir, tmin, tmax} (lbvh.h:388-401)
  hits       HIT_DTYPE [m]    {prim, t, u, v}; miss = {0xffffffff, inf, 0, 0}
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

NODE_DTYPE = np.dtype(
    [("lo", "<f4", (3,)), ("hi", "<f4", (3,)), ("left", "<u4"), ("right", "<u4")]
)
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
SPHERE_HIT_DTYPE = np.dtype(
    [("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("normal", "<f4", (3,)), ("pad", "<f4")]
)
LEAF_BIT = 0x80000000
MISS = 0xFFFFFFFF

_P = ctypes.c_void_p
_S = ctypes.c_size_t


STAGED_REF = os.path.join(os.path.dirname(HERE), "baseline", "_ref")


def ref_dir() -> str:
    """Where the reference's files are compiled from: $LBVH_REF_DIR, else the
    staged copy in baseline/_ref (see stage_ref.sh)."""
    return os.environ.get("LBVH_REF_DIR") or STAGED_REF


def stage_reference() -> None:
    """Copies the reference files libref.so needs into baseline/_ref where a
    reference checkout is present (a no-op elsewhere)."""
    subprocess.run(["sh", os.path.join(HERE, "stage_ref.sh")], check=True)


def build_libs(ref_dir: str | None = None) -> None:
    """Runs oracle/Makefile (liboracle.so, plus _ref/libref.so when the
    reference's files are present: $LBVH_REF_DIR or baseline/_ref)."""
    cmd = ["make", "-s", "-C", HERE]
    if ref_dir:
        cmd.append(f"REF_DIR={ref_dir}")
    subprocess.run(cmd, check=True)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class _Lib:
    def __init__(self, path: str, prefix: str):
        self.path = path
        self.lib = ctypes.CDLL(path)
        self.p = prefix
        f = self._f
        f("make_triangles", None, [_P, _S, _P])
        f("tri_boxes", None, [_P, _S, _P])
        f("centroid_bounds", None, [_P, _S, _S, _P])
        f("curve", None, [_P, _S, _S, _P, _P, _P])
        f("build", ctypes.c_int, [_P, _S, _S, _P])
        f("build_boxes", ctypes.c_int, [_P, _S, _S, _P])

    def _f(self, name, res, args):
        fn = getattr(self.lib, f"{self.p}_{name}")
        fn.restype = res
        fn.argtypes = args
        setattr(self, "_" + name, fn)

    # -- build path -------------------------------------------------------
    def make_triangles(self, verts: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 9)
        out = np.empty((v.shape[0], 12), np.float32)
        self._make_triangles(_ptr(v), v.shape[0], _ptr(out))
        return out

    def tri_boxes(self, tris: np.ndarray) -> np.ndarray:
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        out = np.empty((t.shape[0], 6), np.float32)
        self._tri_boxes(_ptr(t), t.shape[0], _ptr(out))
        return out

    def centroid_bounds(self, tris: np.ndarray, threads: int = 1) -> np.ndarray:
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        out = np.empty(6, np.float32)
        self._centroid_bounds(_ptr(t), t.shape[0], threads, _ptr(out))
        return out

    def curve(self, tris: np.ndarray, threads: int = 1):
        """(codes in input order, sorted codes, stable sort permutation)."""
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        n = t.shape[0]
        codes = np.empty(n, np.uint32)
        scodes = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        self._curve(_ptr(t), n, threads, _ptr(codes), _ptr(scodes), _ptr(perm))
        return codes, scodes, perm

    def build(self, tris: np.ndarray, threads: int = 1) -> np.ndarray:
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        n = t.shape[0]
        if n < 2:
            raise ValueError("the reference build needs at least 2 primitives")
        out = np.zeros(n - 1, NODE_DTYPE)
        rc = self._build(_ptr(t), n, threads, _ptr(out))
        assert rc == 0
        return out

    def build_boxes(self, boxes: np.ndarray, threads: int = 1) -> np.ndarray:
        b = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 6)
        n = b.shape[0]
        if n < 2:
            raise ValueError("the reference build needs at least 2 primitives")
        out = np.zeros(n - 1, NODE_DTYPE)
        rc = self._build_boxes(_ptr(b), n, threads, _ptr(out))
        assert rc == 0
        return out


class Port(_Lib):
    """The C++ restatement (lbvh_oracle.cpp)."""

    def __init__(self, path: str):
        super().__init__(path, "orc")
        f = self._f
        f("split", None, [_P, _S, _P])
        f("refit", ctypes.c_int, [_P, _S, _P])
        f("trace", None, [_P, _P, _P, _S, _S, _P, _P, _P])
        f("check_bvh", ctypes.c_long, [_P, _S])
        f("trace_spheres", None, [_P, _P, _P, _S, _S, _P])

    def split(self, sorted_codes: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(sorted_codes, dtype=np.uint32)
        out = np.empty((max(c.size - 1, 0), 2), np.uint32)
        self._split(_ptr(c), c.size, _ptr(out))
        return out

    def refit(self, nodes: np.ndarray, tris: np.ndarray) -> np.ndarray:
        out = np.array(nodes, dtype=NODE_DTYPE, copy=True)
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        rc = self._refit(_ptr(out), out.size, _ptr(t))
        assert rc == 0
        return out

    def trace(self, nodes, tris, rays, threads: int = 1, counts: bool = False):
        nd = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        m = r.shape[0]
        hits = np.empty(m, HIT_DTYPE)
        nb = np.empty(m, np.uint32) if counts else None
        nt = np.empty(m, np.uint32) if counts else None
        self._trace(_ptr(nd), _ptr(t), _ptr(r), m, threads, _ptr(hits), _ptr(nb), _ptr(nt))
        return (hits, nb, nt) if counts else hits

    def trace_spheres(self, nodes, spheres, rays, threads: int = 1):
        """Closest sphere hits (the example program's intersector) over a
        tree built from the spheres' boxes."""
        nd = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        sp = np.ascontiguousarray(spheres, dtype=np.float32).reshape(-1, 4)
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.empty(r.shape[0], SPHERE_HIT_DTYPE)
        self._trace_spheres(_ptr(nd), _ptr(sp), _ptr(r), r.shape[0], threads, _ptr(hits))
        return hits

    def check_bvh(self, nodes) -> int:
        nd = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        return int(self._check_bvh(_ptr(nd), nd.size))


class Ref(_Lib):
    """The unmodified reference header behind ref_shim.cpp."""

    def __init__(self, path: str):
        super().__init__(path, "ref")
        f = self._f
        f("trace", None, [_P, _S, _P, _S, _P, _S, _S, _P])
        f("load_obj", ctypes.c_long, [ctypes.c_char_p, _P, _S])
        f("trace_spheres", None, [_P, _S, _P, _S, _P, _S, _S, _P])

    def trace(self, nodes, tris, rays, threads: int = 1):
        nd = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 12)
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        m = r.shape[0]
        hits = np.empty(m, HIT_DTYPE)
        self._trace(_ptr(nd), nd.size, _ptr(t), t.shape[0], _ptr(r), m, threads, _ptr(hits))
        return hits

    def trace_spheres(self, nodes, spheres, rays, threads: int = 1):
        nd = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
        sp = np.ascontiguousarray(spheres, dtype=np.float32).reshape(-1, 4)
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.empty(r.shape[0], SPHERE_HIT_DTYPE)
        self._trace_spheres(_ptr(nd), nd.size, _ptr(sp), sp.shape[0], _ptr(r), r.shape[0], threads, _ptr(hits))
        return hits

    def load_obj(self, path: str) -> np.ndarray:
        n = self._load_obj(path.encode(), None, 0)
        if n < 0:
            raise OSError(f"cannot parse {path}")
        out = np.empty((n, 12), np.float32)
        k = self._load_obj(path.encode(), _ptr(out), n)
        return out[:k]


_port = None
_ref = None


def port() -> Port:
    """The restatement; builds liboracle.so on first use if it is missing."""
    global _port
    if _port is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build_libs()
        _port = Port(path)
    return _port


def ref() -> Ref | None:
    """The reference itself, or None where it was not built (no reference
    files were staged on this machine)."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            return None
        _ref = Ref(path)
    return _ref
