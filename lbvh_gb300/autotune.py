"""Autotuner for the GPU launch shapes and sort parameters (results are
unaffected; only speed).

Tunes, on a caller-supplied sample workload:
  * the batched build (tune_batch): its CTA size (LBVH_PARAM_BATCH_THREADS:
    256, 512, 1024 threads), the radix width of its CTA-local sort
    (LBVH_PARAM_BATCH_RADIX_BITS: 4, 6 or 8-bit digits, i.e. 8, 5 or 4 passes)
    and the keys each thread ranks per chunk (LBVH_PARAM_BATCH_KEYS_PER_THREAD:
    4 or 8); then the persistent traversal grid
    (LBVH_PARAM_TRACE_BLOCKS_PER_SM), the ray-refill threshold
    (LBVH_PARAM_TRACE_REFILL) and the leaf-test batching
    (LBVH_PARAM_TRACE_LEAF_BATCH) of the batched trace;
  * the plain trace (tune_trace), per workload: the leaf-test batching
    (LBVH_PARAM_TRACE_LEAF_BATCH) and the ray-refill threshold, timed on a
    sample of the workload's rays -- long rays through loose trees gain from
    batching the triangle tests of a warp's lanes, short rays lose;
  * the handling of page-locked host rays and hits (tune_transfer,
    LBVH_PARAM_TRACE_IN_PLACE), timed on the caller's own buffers;
  * the plain build (tune_build), per size class (primitive counts in
    [2^k, 2^(k+1))): the keys-only sort's tile (LBVH_PARAM_SORT_TILE_KEYS:
    1,024 or 4,096 keys), whether the bucket sort runs
    (LBVH_PARAM_BUCKET_SORT_MIN) and the bounds pass's CTAs per SM
    (LBVH_PARAM_BOUNDS_BLOCKS_PER_SM).
The best setting per workload key is kept in a JSON table (by default
$LBVH_TUNE_CACHE, else ~/.cache/lbvh_gb300/tuning.json) and applied to a
context with apply().
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import _lib

BATCH_THREADS = (256, 512, 1024)
BATCH_RADIX_BITS = (4, 6, 8)
BATCH_KEYS_PER_THREAD = (4, 8)
TRACE_BLOCKS_PER_SM = (6, 8)
TRACE_REFILL = (8, 12, 16)
TRACE_LEAF_BATCH = (1, 4, 8)
TRACE_GRID = (8, 9)  # CTAs per SM; the leaf-batching variant is compiled to fit 9
TRACE_RAY_ORDER = (0, 1)  # the caller's order, sorted by origin and direction cells
SORT_TILE_KEYS = (1024, 4096)
BOUNDS_BLOCKS_PER_SM = (2, 4, 8)
BUCKET_SORT_MIN = 65536  # the smallest size the bucket sort may take
BUCKET_SORT_OFF = 1 << 30  # a threshold no build reaches

# setting key -> context parameter
_PARAMS = {
    "batch_threads": "PARAM_BATCH_THREADS",
    "batch_radix_bits": "PARAM_BATCH_RADIX_BITS",
    "batch_keys_per_thread": "PARAM_BATCH_KEYS_PER_THREAD",
    "trace_blocks_per_sm": "PARAM_TRACE_BLOCKS_PER_SM",
    "trace_refill": "PARAM_TRACE_REFILL",
    "trace_leaf_batch": "PARAM_TRACE_LEAF_BATCH",
    "sort_tile_keys": "PARAM_SORT_TILE_KEYS",
    "bucket_sort_min": "PARAM_BUCKET_SORT_MIN",
    "bounds_blocks_per_sm": "PARAM_BOUNDS_BLOCKS_PER_SM",
    "trace_in_place": "PARAM_TRACE_IN_PLACE",
    "trace_ray_order": "PARAM_TRACE_RAY_ORDER",
}


def size_class(n: int) -> int:
    """The size class of a build of n primitives: k with 2^k <= n < 2^(k+1)."""
    return max(int(n), 1).bit_length() - 1


def build_key(n: int, device: str = "gb300") -> str:
    return f"{device}:build:2^{size_class(n)}"


def cache_path() -> str:
    p = os.environ.get("LBVH_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "lbvh_gb300", "tuning.json")


def load_table(path: str | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            table = json.load(f)
    except (OSError, ValueError):
        return {}
    return table if isinstance(table, dict) else {}  # not a table: start a new one


def save_table(table: dict, path: str | None = None) -> None:
    path = path or cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(ctx, setting: dict) -> None:
    """Sets the context parameters a setting names (other keys -- the
    timings kept beside them -- are ignored)."""
    for key, name in _PARAMS.items():
        if key in setting:
            ctx.set_param(getattr(_lib, name), int(setting[key]))


def apply_build(ctx, n: int, table_path: str | None = None, device: str = "gb300") -> dict | None:
    """Applies the tuned plain-build setting of n's size class, if any."""
    setting = load_table(table_path).get(build_key(n, device))
    if setting:
        apply(ctx, setting)
    return setting


def _time(fn, stream, reps: int) -> float:
    import torch

    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def _store(table, key, setting, table_path):
    table[key] = setting
    try:
        save_table(table, table_path)
    except OSError:
        pass  # a read-only home: keep the setting for this process only


def tune_batch(ctx, tris, offsets, rays, ray_offsets, key: str, reps: int = 3, table_path: str | None = None,
               force: bool = False) -> dict:
    """Best build and trace parameters for a batched build + trace workload
    (device arrays); cached under `key`. Returns the setting and applies
    it."""
    import torch

    from .api import Batch

    table = load_table(table_path)
    if key in table and not force:
        apply(ctx, table[key])
        return table[key]
    stream = torch.cuda.current_stream()
    batch = Batch(ctx)
    out = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=rays.device)
    build_ms = {}
    for t in BATCH_THREADS:
        for bits in BATCH_RADIX_BITS:
            for items in BATCH_KEYS_PER_THREAD:
                apply(ctx, {"batch_threads": t, "batch_radix_bits": bits, "batch_keys_per_thread": items})
                build_ms[(t, bits, items)] = _time(lambda: batch.build(tris, offsets), stream, reps)
    best_t, best_bits, best_items = min(build_ms, key=build_ms.get)
    apply(ctx, {"batch_threads": best_t, "batch_radix_bits": best_bits, "batch_keys_per_thread": best_items})
    batch.build(tris, offsets)
    trace_ms = {}
    for bps in TRACE_BLOCKS_PER_SM:
        for refill in TRACE_REFILL:
            for leaf in TRACE_LEAF_BATCH:
                apply(ctx, {"trace_blocks_per_sm": bps, "trace_refill": refill, "trace_leaf_batch": leaf})
                trace_ms[(bps, refill, leaf)] = _time(lambda: batch.trace(rays, ray_offsets, out=out), stream, reps)
    bps, refill, leaf = min(trace_ms, key=trace_ms.get)
    setting = {"batch_threads": best_t, "batch_radix_bits": best_bits, "batch_keys_per_thread": best_items,
               "trace_blocks_per_sm": bps, "trace_refill": refill, "trace_leaf_batch": leaf,
               "build_ms": {"x".join(map(str, k)): round(v, 4) for k, v in build_ms.items()},
               "trace_ms": {"x".join(map(str, k)): round(v, 4) for k, v in trace_ms.items()}}
    _store(table, key, setting, table_path)
    apply(ctx, setting)
    return setting


def build_candidates(n: int) -> list[dict]:
    """The plain-build settings tried for a build of n primitives."""
    out = []
    for tile in SORT_TILE_KEYS:
        for bounds in BOUNDS_BLOCKS_PER_SM:
            out.append({"sort_tile_keys": tile, "bucket_sort_min": BUCKET_SORT_OFF, "bounds_blocks_per_sm": bounds})
    if n >= BUCKET_SORT_MIN:
        for bounds in BOUNDS_BLOCKS_PER_SM:
            out.append({"sort_tile_keys": 0, "bucket_sort_min": BUCKET_SORT_MIN, "bounds_blocks_per_sm": bounds})
    return out


def tune_build(ctx, tris, reps: int = 5, table_path: str | None = None, force: bool = False,
               device: str = "gb300") -> dict:
    """Best plain-build setting for the size class of `tris` (a device
    triangle array), timed on that array; cached per size class. Returns
    the setting and applies it."""
    import torch

    from .api import BVH, Builder

    n = int(tris.shape[0])
    key = build_key(n, device)
    table = load_table(table_path)
    if key in table and not force:
        apply(ctx, table[key])
        return table[key]
    stream = torch.cuda.current_stream()
    builder, bvh = Builder(ctx), BVH(ctx)
    ms = []
    for cand in build_candidates(n):
        apply(ctx, cand)
        ms.append(_time(lambda: builder(tris, into=bvh), stream, reps))
    best = dict(build_candidates(n)[int(np.argmin(ms))])
    best["build_ms"] = {f"tile{c['sort_tile_keys']}_bucket{int(c['bucket_sort_min'] < BUCKET_SORT_OFF)}"
                        f"_bounds{c['bounds_blocks_per_sm']}": round(t, 4) for c, t in zip(build_candidates(n), ms)}
    best["tuned_on"] = n
    _store(table, key, best, table_path)
    apply(ctx, best)
    return best


def tune_trace(ctx, bvh, rays, key: str, sample: int | None = None, reps: int = 2, table_path: str | None = None,
               force: bool = False) -> dict:
    """Best leaf-test batching, refill threshold, grid and ray order for
    tracing `rays` (a device [m, 8] array, or a list of them traced one after
    another, as a step that traces several ray sets does) against `bvh`;
    cached under `key`. Timed on all the rays by default: a sample too small
    to fill the GPU, or too sparse to keep neighbouring rays together,
    favours other settings than the full workload does. `sample` (a single
    array only) times about that many rays instead, taken as evenly spaced
    runs of 4,096 consecutive rays. Returns the setting and applies it."""
    import torch

    from .api import Traverser

    table = load_table(table_path)
    if key in table and not force:
        apply(ctx, table[key])
        return table[key]
    stream = torch.cuda.current_stream()
    sets = list(rays) if isinstance(rays, (list, tuple)) else [rays]
    if len(sets) == 1 and sample is not None and sample < int(sets[0].shape[0]):
        m = int(sets[0].shape[0])
        run = 4096
        starts = np.linspace(0, m - run, max(1, sample // run)).astype(np.int64) if m > run else np.zeros(1, np.int64)
        sets = [torch.cat([sets[0][int(a):int(a) + run] for a in starts]).contiguous()]
    outs = [torch.empty((r.shape[0], 4), dtype=torch.float32, device=r.device) for r in sets]
    trav = Traverser(bvh)
    ms = {}
    for order in TRACE_RAY_ORDER:
        for leaf in TRACE_LEAF_BATCH:
            for refill in TRACE_REFILL:
                for grid in TRACE_GRID if leaf > 1 else TRACE_GRID[:1]:
                    apply(ctx, {"trace_leaf_batch": leaf, "trace_refill": refill, "trace_blocks_per_sm": grid,
                                "trace_ray_order": order})
                    ms[(leaf, refill, grid, order)] = _time(lambda: [trav(r, out=o) for r, o in zip(sets, outs)],
                                                            stream, reps)
    leaf, refill, grid, order = min(ms, key=ms.get)
    setting = {"trace_leaf_batch": leaf, "trace_refill": refill, "trace_blocks_per_sm": grid,
               "trace_ray_order": order, "sample_rays": int(sum(int(r.shape[0]) for r in sets)),
               "trace_ms": {"x".join(map(str, k)): round(v, 4) for k, v in ms.items()}}
    _store(table, key, setting, table_path)
    apply(ctx, setting)
    return setting


TRACE_IN_PLACE = (0, 1, 2)


def tune_transfer(ctx, bvh, pairs, key: str, reps: int = 2, table_path: str | None = None,
                  force: bool = False) -> dict:
    """Best handling of host rays and hits (LBVH_PARAM_TRACE_IN_PLACE: 0
    copies both, 1 reads the rays in place and copies the hits back, 2 also
    writes the hits in place) for tracing page-locked host ray arrays
    against `bvh`: `pairs` is a list of (rays, hits) host arrays traced one
    after the other, as the caller's step does. Long traces favour copying
    the hits back once; short ones favour writing them in place. Cached
    under `key`; returns the setting and applies it."""
    import time

    from .api import Traverser

    table = load_table(table_path)
    if key in table and not force:
        apply(ctx, table[key])
        return table[key]
    trav = Traverser(bvh)
    ms = {}
    for mode in TRACE_IN_PLACE:
        ctx.set_param(_lib.PARAM_TRACE_IN_PLACE, mode)
        for r, h in pairs:  # first touch of this mode's paths
            trav(r, out=h)
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            for r, h in pairs:
                trav(r, out=h)  # host buffers: each call returns finished
            ts.append(1e3 * (time.perf_counter() - t0))
        ms[mode] = float(np.median(ts))
    best = min(ms, key=ms.get)
    setting = {"trace_in_place": best, "host_trace_ms": {str(k): round(v, 4) for k, v in ms.items()}}
    _store(table, key, setting, table_path)
    apply(ctx, setting)
    return setting
