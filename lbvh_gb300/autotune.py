"""Autotuner for the GPU launch shapes (results are unaffected; only speed).

Tunes, on a caller-supplied sample workload:
  * the CTA size of the batched build (LBVH_PARAM_BATCH_THREADS: 256, 512,
    1024 threads; each sort chunk is CTA size x 4 keys, 8-bit radix digits);
  * the persistent traversal grid (LBVH_PARAM_TRACE_BLOCKS_PER_SM) and the
    ray-refill threshold (LBVH_PARAM_TRACE_REFILL).
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
TRACE_BLOCKS_PER_SM = (6, 8)
TRACE_REFILL = (8, 12, 16)


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
    if "batch_threads" in setting:
        ctx.set_param(_lib.PARAM_BATCH_THREADS, int(setting["batch_threads"]))
    if "trace_blocks_per_sm" in setting:
        ctx.set_param(_lib.PARAM_TRACE_BLOCKS_PER_SM, int(setting["trace_blocks_per_sm"]))
    if "trace_refill" in setting:
        ctx.set_param(_lib.PARAM_TRACE_REFILL, int(setting["trace_refill"]))


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


def tune_batch(ctx, tris, offsets, rays, ray_offsets, key: str, reps: int = 3, table_path: str | None = None,
               force: bool = False) -> dict:
    """Best launch shapes for a batched build + trace workload (device
    arrays); cached under `key`. Returns the setting and applies it."""
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
        ctx.set_param(_lib.PARAM_BATCH_THREADS, t)
        build_ms[t] = _time(lambda: batch.build(tris, offsets), stream, reps)
    best_t = min(build_ms, key=build_ms.get)
    ctx.set_param(_lib.PARAM_BATCH_THREADS, best_t)
    batch.build(tris, offsets)
    trace_ms = {}
    for bps in TRACE_BLOCKS_PER_SM:
        for refill in TRACE_REFILL:
            ctx.set_param(_lib.PARAM_TRACE_BLOCKS_PER_SM, bps)
            ctx.set_param(_lib.PARAM_TRACE_REFILL, refill)
            trace_ms[(bps, refill)] = _time(lambda: batch.trace(rays, ray_offsets, out=out), stream, reps)
    bps, refill = min(trace_ms, key=trace_ms.get)
    setting = {"batch_threads": best_t, "trace_blocks_per_sm": bps, "trace_refill": refill,
               "build_ms": {str(k): round(v, 4) for k, v in build_ms.items()},
               "trace_ms": {f"{k[0]}x{k[1]}": round(v, 4) for k, v in trace_ms.items()}}
    table[key] = setting
    try:
        save_table(table, table_path)
    except OSError:
        pass  # a read-only home: keep the setting for this process only
    apply(ctx, setting)
    return setting
