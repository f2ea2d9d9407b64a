"""LBVH build + closest-hit trace benchmark on one GB300 (or N replicas).

Default workload (one "step"), the large clustered scene: a room of 262,267
triangles (walls, 64 columns, 500 clutter clusters; generation order kept,
so leaf p is primitive p as in the reference) is built from device-resident
triangles, then traced with 1920 x 1080 primary rays from a pinhole camera
and with one cosine-weighted diffuse bounce ray per primary hit. The bounce
rays are made once, before timing, from the primary hits (bit-identical on
both arms), so every step traces the same 4.1M rays. `value` is rays per
second over whole steps (build included), in Mrays/s; `build` and `trace`
give the stages alone. The L2 (129 MB) is flushed by writing a 256 MB buffer
between timed steps, outside the timing.

Also measured (not part of the step): `e2e`, the same step through the
public API from page-locked host buffers; the build of a 16M-triangle random
soup, the workload of the HBM roofline (`build_16m`, with a refit; the
headline `roofline`); the mid-size torus step (`config1`); 4,096 meshes
built and traced as one batch against the plain per-mesh path (`batched`);
and Poisson request streams through the request server against the plain
path (`served`). Full records of those sections are printed as `detail`
lines before the final line, which carries their summaries.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the unmodified reference (lbvh::builder<float> and
lbvh::traverser, compiled from the staged reference files into
oracle/_ref/libref.so; the bit-exact restatement only where they are absent)
on the same step, the same rays, all host cores.

Under torchrun (N > 1) every rank runs an independent replica of the same
step on its own GPU ("replicas only": the path has no exchange step); value
is the sum of rays over all ranks / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Build Mprims/s + trace Mrays/s (1 GB300)"
WORKLOAD = "room262267_primary1920x1080_diffusebounce"
CONFIG1_WORKLOAD = "torus8320_primary1024x1024_incoherent1M"
L2_POLICY = "GPU arm: L2 flushed (256 MB write) between timed steps"
LEAF_ORDER = "reference parity (leaf p = primitive p)"
N_BUILD_16M = 16_000_000
# Algorithmic HBM bytes per primitive of an LBVH build, by stage: the fixed
# yardstick of the roofline (read the 36 used bytes of a triangle for the
# bounds, again for the Morton code + write an 8-byte entry, four 8-bit sort
# passes over 8-byte entries + histograms, the split's code read and child /
# parent writes, the fit's leaf, child-box, node and flag traffic).
BYTES_PER_PRIM = {"bounds": 36, "morton": 44, "sort": 68, "split": 20, "fit": 96}  # 264 in all


def measured_traffic(key: str, field: str):
    """DRAM bytes (read + write) of one launch / build from the committed
    ncu capture summarised in profiles/ (traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return int(json.load(f)[key][field])
    except (OSError, KeyError, ValueError):
        return None


def measured_profile(key: str, fields):
    """Figures of one kernel's committed ncu capture (profiles/traffic.json),
    with the summary they come from; None when absent."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)[key]
        out = {k: d[k] for k in fields if k in d}
        return dict(out, source="profiles/" + d["summary"]) if out else None
    except (OSError, KeyError, ValueError):
        return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def mark(self, begin: bool):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        inside = [s for t, s in self.samples if self.t0 and self.t1 and self.t0 - 0.05 <= t <= self.t1 + 0.05]
        if not inside and self.samples:  # timed region shorter than one sample period
            mid = 0.5 * ((self.t0 or 0) + (self.t1 or 0))
            inside = [min(self.samples, key=lambda ts: abs(ts[0] - mid))[1]]
        sm, mx, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in inside:
            f = [x.strip() for x in s.split(",")]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except Exception:
                continue
            for k, name in enumerate(names[1:], start=5):
                if k < len(f) and f[k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(inside)}


def replica_throughput(step_ms: float, units: int, world: int, device=None):
    """Whole-job throughput of `world` independent replicas, each
    processing `units` per step: the slowest rank's step time (max over
    ranks) and units x world / that time, in millions per second."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([step_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    return step_ms, world * units / (step_ms * 1e-3) / 1e6


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# --------------------------------------------------------------------------
# reference arm: the reference's CPU implementation on the host cores


def room_workload():
    """The large clustered scene and its primary rays: 262,267 triangles,
    1920 x 1080 pinhole rays from inside the room."""
    from lbvh_gb300 import scenes

    tris = scenes.room_scene(seed=21)
    prim = scenes.pinhole_rays(1920, 1080, eye=(0.0, 3.0, 9.0), target=(0.0, 2.0, 0.0))
    return tris, prim


def room_bounce(prim, hits, tris):
    """One cosine-weighted diffuse bounce ray per primary hit."""
    from lbvh_gb300 import scenes

    return scenes.diffuse_bounce(prim, hits, tris, seed=22)


def room_config(tris, prim, bounce, world):
    """The step's config, identical on both arms (the digest covers every
    ray the step traces)."""
    import hashlib

    h = hashlib.sha1(prim.tobytes())
    h.update(bounce.tobytes())
    return {"workload": WORKLOAD, "triangles": int(tris.shape[0]), "primary_rays": int(prim.shape[0]),
            "bounce_rays": int(bounce.shape[0]), "rays_per_step": int(prim.shape[0] + bounce.shape[0]),
            "rays_sha1": h.hexdigest()[:16], "parallelism": f"replicas{world}", "l2": L2_POLICY,
            "leaf_order": LEAF_ORDER}


def cpu_impl():
    """The reference's own CPU builder and traverser (oracle/_ref/libref.so,
    compiled from the unmodified reference header), else the bit-exact port."""
    import oracle

    impl = oracle.ref()
    if impl is not None:
        return impl, "reference", impl.path
    impl = oracle.port()
    return impl, "port", impl.path


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    impl, kind, path = cpu_impl()
    cores = os.cpu_count() or 1
    tris, prim = room_workload()
    nodes = impl.build(tris, cores)
    bounce = room_bounce(prim, impl.trace(nodes, tris, prim, cores), tris)
    m = prim.shape[0] + bounce.shape[0]
    # warm-up steps: the whole build, rays sampled (nothing on the CPU warms
    # up beyond first-touch of the buffers)
    for _ in range(args.warmup):
        nodes = impl.build(tris, cores)
        impl.trace(nodes, tris, prim[::64], cores)
        impl.trace(nodes, tris, bounce[::64], cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        nodes = impl.build(tris, cores)
        impl.trace(nodes, tris, prim, cores)
        impl.trace(nodes, tris, bounce, cores)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(times))
    value = m / (ms * 1e-3) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": room_config(tris, prim, bounce, world),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": cores, "kind": kind,
                         "lib": os.path.relpath(path, ROOT),
                         "sample": f"the whole step: build of all {tris.shape[0]} triangles + all {m} rays"},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_build_16m(ctx, builder, stream, flush, dev, steps, hbm_peak, peak_kind, n=N_BUILD_16M, span=1.0,
                      with_refit=False):
    """Device-resident build of the 16M-triangle random soup, L2 flushed
    between builds; the HBM roofline workload. span > 1 (profiling) turns
    two triangles into points at -span and +span on every axis, so that the
    soup fills fewer, denser cells of the Morton grid: a smaller soup then
    has the per-bucket occupancy of the full-size one."""
    import torch

    import lbvh_gb300 as lb
    from lbvh_gb300 import scenes

    from lbvh_gb300 import autotune

    host = scenes.soup_large(n, seed=16)
    if span != 1.0:
        host[0] = -span
        host[1] = span
    soup = torch.from_numpy(host).to(dev)
    big = lb.BVH(ctx)
    ctx.reserve(n, 0)
    tuning = autotune.tune_build(ctx, soup)  # this size class's sort / bounds setting
    for _ in range(3):
        builder(soup, into=big)
    torch.cuda.synchronize()
    bt = []
    for _ in range(max(5, min(steps, 20))):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        builder(soup, into=big)
        b.record(stream)
        torch.cuda.synchronize()
        bt.append(a.elapsed_time(b))
    ctx.synchronize()
    ms16 = float(np.mean(bt))
    refit_ms = None
    if with_refit:  # the same tree over moved triangles (topology kept)
        moved = soup + 0.001
        big.refit(moved)
        torch.cuda.synchronize()
        rt = []
        for _ in range(max(5, min(steps, 20))):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            big.refit(moved)
            b.record(stream)
            torch.cuda.synchronize()
            rt.append(a.elapsed_time(b))
        refit_ms = round(float(np.mean(rt)), 4)
        del moved
    algo = n * sum(BYTES_PER_PRIM.values())
    achieved = algo / (ms16 * 1e-3) / 1e9
    return {"triangles": n, "ms": round(ms16, 4),
            "mprims_s": round(n / (ms16 * 1e-3) / 1e6, 1),
            "refit_ms": refit_ms,
            "tuning": tuning,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                         "bytes_per_prim": sum(BYTES_PER_PRIM.values()),
                         "traffic": measured_traffic("build_16m", "dram_bytes_per_build") if n == N_BUILD_16M else None,
                         "traffic_scope": "DRAM bytes of one whole build (all kernels), ncu",
                         "peak_kind": peak_kind}}


def _pct(xs, q):
    return round(1e3 * float(np.percentile(np.asarray(xs), q)), 3) if len(xs) else None


SERVE_SLOTS = 16  # worker streams of the request server


class _PinnedArena:
    """One page-locked host allocation that request arrays and hit buffers
    are carved from (256-byte aligned), as a serving front end's pooled I/O
    buffers are."""

    def __init__(self, nbytes):
        import torch

        self._t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, pin_memory=True)
        self._a = self._t.numpy()
        self._off = 0

    def take(self, nbytes):
        assert self._off + nbytes <= self._a.shape[0]
        v = self._a[self._off : self._off + nbytes]
        self._off += (nbytes + 255) & ~255
        return v


def _owner(a):
    while isinstance(a.base, np.ndarray):
        a = a.base
    return a


def _pinned_requests(reqs):
    """The same requests with every data array moved into one page-locked
    arena (views keep their offsets within a shared array, so ray slices of
    one pooled ray set stay slices of one pinned copy), and room for both
    paths' hit buffers. Returns (arena, requests)."""
    owners = {}
    for _, _, _, d in reqs:
        o = _owner(d)
        assert o.flags.c_contiguous and d.flags.c_contiguous
        owners.setdefault(id(o), o)
    hit_bytes = sum(d.shape[0] * 16 for _, k, _, d in reqs if k == "trace")
    size = sum((o.nbytes + 255) & ~255 for o in owners.values()) + 2 * (hit_bytes + 256 * len(reqs))
    arena = _PinnedArena(size)
    copies = {}
    for key, o in owners.items():
        p = arena.take(o.nbytes)
        p[:] = o.reshape(-1).view(np.uint8)
        copies[key] = (o, p)
    out, views = [], {}
    for at, kind, scene, d in reqs:
        if id(d) not in views:
            o, p = copies[id(_owner(d))]
            off = d.__array_interface__["data"][0] - o.__array_interface__["data"][0]
            views[id(d)] = p[off : off + d.nbytes].view(d.dtype).reshape(d.shape)
        out.append((at, kind, scene, views[id(d)]))
    return arena, out


def _result_buffers(reqs, device, arena=None):
    """One hit buffer per trace request, already mapped for device copies
    (as a serving front end's pooled response buffers are); carved from
    `arena` when given."""
    import torch

    import lbvh_gb300 as lb

    def hits(m):
        if arena is None:
            return np.empty(m, lb.HIT_DTYPE)
        return arena.take(16 * m).view(lb.HIT_DTYPE)

    outs = [hits(d.shape[0]) if k == "trace" else None for _, k, _, d in reqs]
    zeros = torch.zeros((max([o.shape[0] for o in outs if o is not None] + [1]), 4), device=device)
    for o in outs:
        if o is not None and o.shape[0]:
            torch.from_numpy(o.view(np.float32).reshape(-1, 4)).copy_(zeros[: o.shape[0]])
    return outs


def _served_run(reqs, device, slots=SERVE_SLOTS, buffers="pageable"):
    """One arrival stream through the request server and through the plain
    API; latency from each request's (nominal) arrival. Both paths write
    trace hits into caller-provided, already mapped result buffers; with
    buffers="pinned" the request arrays and the hit buffers of both paths
    are page-locked host memory (one arena), else pageable arrays."""
    import torch

    from lbvh_gb300 import scenes
    from lbvh_gb300.serve import Server, run_plain

    arena = None
    if buffers == "pinned":
        try:
            arena, reqs = _pinned_requests(reqs)
        except RuntimeError as e:  # the host would not lock that much memory
            buffers = "pageable (page-locking failed: " + str(e).splitlines()[0][:120] + ")"
    # every request array is copied to the device once before either path
    # runs, so neither pays the first device access to its pages
    seen = set()
    for _, _, _, data in reqs:
        if id(data) not in seen:
            seen.add(id(data))
            torch.from_numpy(np.ascontiguousarray(data)).to(device)
    outs_srv = _result_buffers(reqs, device, arena)
    outs_plain = _result_buffers(reqs, device, arena)
    torch.cuda.synchronize()
    with Server(device, slots=slots, hbm_budget=120 << 30) as srv:
        srv.submit("build", -1, scenes.soup(1000, 1)).result()  # library warm-up
        srv.submit("trace", -1, scenes.pinhole_rays(64, 64)).result()
        srv.done.clear()
        futs = []
        t0 = time.perf_counter()
        s0 = srv.clock()  # the same instant on the server's clock
        for at, kind, scene, data in reqs:
            wait = t0 + at - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            futs.append(srv.submit(kind, scene, data, out=outs_srv[len(futs)]))
        results = [f.result(timeout=600) for f in futs]
        done = {id(r.future): r for r in srv.done}
        coalesced, evictions = srv.coalesced, srv.evictions
    # latency from the nominal arrival time (a submit that ran late because
    # the producer fell behind still counts from when it was due)
    recs = [(at, kind, done[id(f)]) for (at, kind, _, _), f in zip(reqs, futs)]
    lat = [r.done - (s0 + at) for at, _, r in recs]
    span = max(r.done for _, _, r in recs) - (s0 + reqs[0][0])
    by_kind = {}
    for (at, kind, r), x in zip(recs, lat):
        by_kind.setdefault(kind, []).append(x)
    plain = run_plain(reqs, device, outs=outs_plain)
    plat = [x[1] for x in plain]
    pspan = max(at + l for (at, _, _, _), l in zip(reqs, plat)) - reqs[0][0]
    bad = [i for i, (a, (b, _)) in enumerate(zip(results, plain))
           if not (a is None and b is None or (a is not None and b is not None and a.tobytes() == b.tobytes()))]
    rays = sum(d.shape[0] for _, k, _, d in reqs if k == "trace")
    del results, plain
    torch.cuda.empty_cache()
    kinds = [k for _, k, _, _ in reqs]
    out = {"requests": len(reqs), "mix": {k: kinds.count(k) for k in ("build", "refit", "trace")},
           "worker_streams": slots, "results": "caller-provided hit buffers, mapped before the run (both paths)",
           "host_buffers": buffers,
           "server": {"p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99), "throughput_req_s": round(len(lat) / span, 1),
                      "trace_mrays_s": round(rays / span / 1e6, 1), "coalesced_requests": coalesced,
                      "evictions": evictions,
                      "by_kind": {k: {"p50_ms": _pct(v, 50), "p99_ms": _pct(v, 99)} for k, v in by_kind.items()}},
           "plain": {"p50_ms": _pct(plat, 50), "p99_ms": _pct(plat, 99),
                     "throughput_req_s": round(len(plat) / pspan, 1), "trace_mrays_s": round(rays / pspan / 1e6, 1)},
           "results_equal": not bad}
    out["throughput_ratio"] = round(out["server"]["throughput_req_s"] / out["plain"]["throughput_req_s"], 2)
    if bad:
        out["mismatched"] = [[i, reqs[i][1], reqs[i][2]] for i in bad[:8]]
    return out


def measure_served(device, seed=7, buffers="pinned"):
    """Served workloads (Poisson arrivals of build / refit / trace requests on
    48 resident scenes, 70% trace / 20% refit / 10% rebuild after one build
    per scene) through the request server (16 worker streams, coalescing,
    120 GB HBM budget), against the same arrivals through the plain API one request at a
    time:
      mix:   scenes 1k-2M triangles, traces 16k-2M rays, 400 requests at
             2,000 requests/s;
      small: scenes 1k-64k triangles, traces 16k-64k rays, 2,000 requests at
             200,000 requests/s (a burst: both paths saturated).
    `buffers` picks the host memory of the request arrays and hit buffers
    (the same for both paths): one "pinned" arena (the default, as a serving
    front end's pooled I/O buffers are) or "pageable" arrays."""
    from lbvh_gb300 import scenes

    mix = scenes.served_requests(400, 2000.0, seed, n_scenes=48)
    out = {"mix": dict(rate_per_s=2000.0, scenes=48, **_served_run(mix, device, buffers=buffers))}
    del mix
    small = scenes.served_requests(2000, 200000.0, seed + 1, n_scenes=48, lo=1000, hi=65536, ray_lo=16384,
                                   ray_hi=65536)
    out["small"] = dict(rate_per_s=200000.0, scenes=48, **_served_run(small, device, buffers=buffers))
    import torch

    if hasattr(torch._C, "_host_emptyCache"):
        torch._C._host_emptyCache()  # hand the pinned arenas' pages back
    return out


def measure_batched(ctx_device, steps, hbm_peak, peak_kind, n_meshes=4096, rays_per_mesh=4096, seed=3):
    """Batched workload: n_meshes soups with log-uniform [64, 65,536]
    triangles and rays_per_mesh random rays each. Build + trace of all meshes
    in one persistent launch each, tuned by the autotuner and replayed as a
    CUDA graph, against the plain path (one build + one trace call per mesh)."""
    import torch

    import lbvh_gb300 as lb
    from lbvh_gb300 import autotune, scenes

    dev = torch.device("cuda", ctx_device)
    tris_h, off_h, rays_h, roff_h = scenes.batch_scene(n_meshes, 64, 65536, rays_per_mesh, seed)
    tris = torch.from_numpy(tris_h).to(dev)
    rays = torch.from_numpy(rays_h).to(dev)
    off = torch.from_numpy(off_h.view(np.int32)).to(dev)
    roff = torch.from_numpy(roff_h.view(np.int32)).to(dev)
    del tris_h, rays_h
    out = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=dev)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    s = torch.cuda.Stream(dev)
    ctx = lb.Context(ctx_device, s.cuda_stream)
    res = {"meshes": n_meshes, "triangles": int(off_h[-1]), "rays": int(rays.shape[0]),
           "workload": f"batch{n_meshes}_loguniform64-65536_{rays_per_mesh}rays"}
    with torch.cuda.stream(s):
        setting = autotune.tune_batch(ctx, tris, off, rays, roff, key=f"gb300:{res['workload']}")
        res["tuning"] = {k: setting[k] for k in ("batch_threads", "batch_radix_bits", "batch_keys_per_thread",
                                                 "trace_blocks_per_sm", "trace_refill", "trace_leaf_batch")}
        batch = lb.Batch(ctx)
        for _ in range(3):
            batch.build(tris, off)
            batch.trace(rays, roff, out=out)
        torch.cuda.synchronize()
        ref_out = out.clone()
        bt, tt = [], []
        for _ in range(max(3, min(steps, 10))):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(s)
            batch.build(tris, off)
            e[1].record(s)
            batch.trace(rays, roff, out=out)
            e[2].record(s)
            torch.cuda.synchronize()
            bt.append(e[0].elapsed_time(e[1]))
            tt.append(e[1].elapsed_time(e[2]))
        ctx.synchronize()
        assert torch.equal(out.view(torch.int32), ref_out.view(torch.int32))
    build_ms, trace_ms = float(np.mean(bt)), float(np.mean(tt))
    res.update({"build_ms": round(build_ms, 3), "trace_ms": round(trace_ms, 3),
                "step_ms": round(build_ms + trace_ms, 3),
                "build_mprims_s": round(res["triangles"] / (build_ms * 1e-3) / 1e6, 1),
                "trace_mrays_s": round(res["rays"] / (trace_ms * 1e-3) / 1e6, 1),
                "gpu_launches_per_step": 5})
    # the same step captured once as a CUDA graph and replayed
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
            batch.build(tris, off)
            batch.trace(rays, roff, out=out)
        gt = []
        for _ in range(max(3, min(steps, 10))):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                a.record(s)
                g.replay()
                b.record(s)
            torch.cuda.synchronize()
            gt.append(a.elapsed_time(b))
        assert torch.equal(out.view(torch.int32), ref_out.view(torch.int32))
        res["graph_step_ms"] = round(float(np.mean(gt)), 3)
    except Exception as exc:  # capture is an optimisation: report why it was skipped
        res["graph_step_ms"] = None
        res["graph_error"] = str(exc)[:200]
    # plain path: one build + one trace call per mesh on the same data
    with torch.cuda.stream(s):
        builder = lb.Builder(ctx)
        bvh = lb.BVH(ctx)
        hits = torch.empty((rays_per_mesh, 4), dtype=torch.float32, device=dev)
        ctx.reserve(65536, 0)
        for k in range(8):  # warm-up
            builder(tris[int(off_h[k]):int(off_h[k + 1])], into=bvh)
            lb.Traverser(bvh)(rays[int(roff_h[k]):int(roff_h[k + 1])], out=hits)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for k in range(n_meshes):
            builder(tris[int(off_h[k]):int(off_h[k + 1])], into=bvh)
            lb.Traverser(bvh)(rays[int(roff_h[k]):int(roff_h[k + 1])], out=hits)
        b.record(s)
        torch.cuda.synchronize()
        plain_ms = max(a.elapsed_time(b), 1e3 * (time.perf_counter() - t0))
    res["plain_step_ms"] = round(plain_ms, 3)
    best = res["graph_step_ms"] or res["step_ms"]
    res["speedup_vs_plain"] = round(plain_ms / best, 2)
    # the same meshes with sorted leaves (each mesh's leaves in stable Morton
    # order): the intended LBVH, whose trees stay tight for randomly ordered
    # input; hits are checked against the plain sorted-leaf path on a sample
    with torch.cuda.stream(s):
        sb = lb.Batch(ctx)
        sout = torch.empty_like(out)
        for _ in range(3):
            sb.build(tris, off, sorted_leaves=True)
            sb.trace(rays, roff, out=sout)
        torch.cuda.synchronize()
        sbt, stt = [], []
        for _ in range(max(3, min(steps, 10))):
            flush.zero_()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(s)
            sb.build(tris, off, sorted_leaves=True)
            e[1].record(s)
            sb.trace(rays, roff, out=sout)
            e[2].record(s)
            torch.cuda.synchronize()
            sbt.append(e[0].elapsed_time(e[1]))
            stt.append(e[1].elapsed_time(e[2]))
        sbuilder = lb.Builder(ctx, sorted_leaves=True)
        for k in range(0, n_meshes, max(1, n_meshes // 16)):
            r0, r1 = int(roff_h[k]), int(roff_h[k + 1])
            want = lb.Traverser(sbuilder(tris[int(off_h[k]):int(off_h[k + 1])]))(rays[r0:r1])
            torch.cuda.synchronize()
            assert torch.equal(want.view(torch.int32), sout[r0:r1].view(torch.int32))
    sbm, stm = float(np.mean(sbt)), float(np.mean(stt))
    res["sorted_leaves"] = {"build_ms": round(sbm, 3), "trace_ms": round(stm, 3), "step_ms": round(sbm + stm, 3),
                            "trace_mrays_s": round(res["rays"] / (stm * 1e-3) / 1e6, 1)}
    del tris, rays, out, flush
    torch.cuda.empty_cache()
    return res


# --------------------------------------------------------------------------
# our arm


TRANSFER_NOTE = {0: "triangles, rays and hits copied (page-locked host buffers)",
                 1: "triangles copied; rays read in place in page-locked host memory, hits copied back",
                 2: "triangles copied; rays read and hits written in place in page-locked host memory"}


def ctx_in_place(ctx, transfer, args):
    """The host-transfer mode the e2e steps ran with."""
    return args.e2e_in_place if args.e2e_in_place is not None else transfer["trace_in_place"]


def build_launches(n, tuning):
    """Kernel launches of one keys-only build of n primitives: one cluster
    launch up to 16,384; else bounds, Morton codes, the bucket sort's three
    kernels when it runs, the four onesweep passes, the local tree phase and
    the merge levels (as the library lays them out)."""
    if n <= 16384:
        return 1
    groups, merges, level = -(-n // 1024), 0, 0
    while groups > 1:
        window = groups if groups <= (160 if level == 0 else 16) else (128 if level == 0 else 16)
        groups = -(-groups // window)
        merges += 1
        level += 1
    bucket = n >= int(tuning.get("bucket_sort_min", 1_500_000))
    return 2 + (3 if bucket else 0) + 4 + 1 + merges


def step_launches(n, tuning, trace_tuning, traces=2):
    """Kernel launches of one bench step: the build, the traversal copy
    (k_repack) and each trace (with the ray order: the key kernel and three
    sort passes before it)."""
    per_trace = 1 + (4 if trace_tuning.get("trace_ray_order") else 0)
    return build_launches(n, tuning) + 1 + traces * per_trace


def time_steps(builder, bvh, trav, tris, ray_sets, hit_sets, flush, stream, steps):
    """K whole steps (build, then one trace per ray set) timed with CUDA
    events on the launching stream, L2 flushed before each step. Returns
    per-step (build ms, trace ms)."""
    import torch

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2 + len(ray_sets))] for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        builder(tris, into=bvh)
        ev[i][1].record(stream)
        for k, (r, h) in enumerate(zip(ray_sets, hit_sets)):
            trav(r, out=h)
            ev[i][2 + k].record(stream)
    torch.cuda.synchronize()
    return [(e[0].elapsed_time(e[1]), e[1].elapsed_time(e[-1])) for e in ev]


def measure_config1(ctx, stream, flush, dev, steps):
    """The mid-size coherent scene (8,320 triangles: torus + ground plane),
    1024 x 1024 primary + 1,048,576 incoherent rays, build included."""
    import torch

    import lbvh_gb300 as lb
    from lbvh_gb300 import scenes

    tris_h = scenes.torus_scene(seed=11)
    rays_h = np.concatenate([scenes.pinhole_rays(1024, 1024), scenes.incoherent_rays(tris_h, 1 << 20, 3)])
    tris = torch.from_numpy(tris_h).to(dev)
    rays = torch.from_numpy(rays_h).to(dev)
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=dev)
    from lbvh_gb300 import autotune

    tuning = autotune.tune_build(ctx, tris)  # this size class's sort / bounds setting
    builder, bvh = lb.Builder(ctx), lb.BVH(ctx)
    builder(tris, into=bvh)
    trace_tuning = autotune.tune_trace(ctx, bvh, rays, key=f"gb300:trace:{CONFIG1_WORKLOAD}")
    trav = lb.Traverser(bvh)
    for _ in range(3):
        builder(tris, into=bvh)
        trav(rays, out=hits)
    t = time_steps(builder, bvh, trav, tris, [rays], [hits], flush, stream, steps)
    b, tr = float(np.mean([x for x, _ in t])), float(np.mean([y for _, y in t]))
    m = rays.shape[0]
    return {"workload": CONFIG1_WORKLOAD, "triangles": int(tris_h.shape[0]), "rays_per_step": int(m),
            "value": round(m / ((b + tr) * 1e-3) / 1e6, 1), "unit": "Mrays/s", "ms_per_step": round(b + tr, 4),
            "build_ms": round(b, 4), "trace_ms": round(tr, 4),
            "tuning": {k: tuning[k] for k in ("sort_tile_keys", "bucket_sort_min", "bounds_blocks_per_sm")},
            "trace_tuning": {k: trace_tuning.get(k, 0) for k in ("trace_leaf_batch", "trace_refill", "trace_blocks_per_sm",
                                                                 "trace_ray_order")}}


def summary_line(line):
    """The final JSON line: the contract's keys plus one-line summaries of
    the extra sections (their full records are the detail lines above)."""
    out = {k: v for k, v in line.items() if k not in ("build_16m", "batched", "served", "config1")}
    b16 = line.get("build_16m")
    if b16:
        out["build_16m"] = {"ms": b16["ms"], "mprims_s": b16["mprims_s"], "refit_ms": b16["refit_ms"],
                            "frac": b16["roofline"]["frac"]}
        t16 = b16.get("tuning") or {}
        out["build_16m"]["tuning"] = [t16.get(k) for k in ("sort_tile_keys", "bucket_sort_min", "bounds_blocks_per_sm")]
    c1 = line.get("config1")
    if c1:
        out["config1"] = {k: c1[k] for k in ("value", "ms_per_step", "build_ms", "trace_ms")}
    bt = line.get("batched")
    if bt:
        out["batched"] = {"graph_step_ms": bt.get("graph_step_ms"), "plain_step_ms": bt["plain_step_ms"],
                          "speedup_vs_plain": bt["speedup_vs_plain"],
                          "sorted_leaves_step_ms": bt["sorted_leaves"]["step_ms"],
                          "tuning": [bt["tuning"].get(k) for k in ("batch_threads", "batch_radix_bits",
                                                                     "batch_keys_per_thread")]}
    sv = line.get("served")
    if sv:
        out["served"] = {k: {"ratio": v["throughput_ratio"], "p99_ms": [v["server"]["p99_ms"], v["plain"]["p99_ms"]],
                             "equal": v["results_equal"]} for k, v in sv.items()}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-16m", action="store_true", help="skip the 16M-triangle build measurement")
    ap.add_argument("--only-16m", action="store_true", help="only the 16M-triangle build (profiling)")
    ap.add_argument("--soup-n", type=int, default=N_BUILD_16M, help="soup size of the build measurement")
    ap.add_argument("--soup-span", type=float, default=1.0,
                    help="profiling: stretch the soup's bounds to +-span (denser Morton buckets)")
    ap.add_argument("--only-step", action="store_true", help="only the headline step (profiling)")
    ap.add_argument("--step-rays", type=int, default=0,
                    help="profiling: trace only every k-th ray of the headline step (0: all)")
    ap.add_argument("--no-config1", action="store_true", help="skip the mid-size torus step")
    ap.add_argument("--only-config1", action="store_true", help="only the mid-size torus step (profiling)")
    ap.add_argument("--tree-walk-fused", type=int, default=None,
                    help="1: walk tree nodes crossing CTA edges from the local phase's tail (default: the library's)")
    ap.add_argument("--small-build-max", type=int, default=None,
                    help="largest build run as one cluster launch, 0 = never (default: the library's)")
    ap.add_argument("--trace-ray-order", type=int, default=None,
                    help="1: traverse the rays in sorted order (default: the tuner's choice)")
    ap.add_argument("--trace-refill", type=int, default=None,
                    help="idle lanes at which a traversal warp takes new rays (default: the library's)")
    ap.add_argument("--trace-blocks", type=int, default=None,
                    help="resident traversal CTAs per SM (default: the library's)")
    ap.add_argument("--e2e-in-place", type=int, default=None,
                    help="host rays / hits of the e2e step: 0 copied in chunks, 1 rays in place, 2 both in place")
    ap.add_argument("--e2e-chunk", type=int, default=None,
                    help="rays per chunk of the e2e step's copied traces (0: one piece)")
    ap.add_argument("--trace-leaf-batch", type=int, default=None,
                    help="lanes with pending triangle tests before a traversal warp runs them (default: the library's)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-meshes measurement")
    ap.add_argument("--only-batched", action="store_true", help="only the batched-meshes measurement")
    ap.add_argument("--no-served", action="store_true", help="skip the served-requests measurement")
    ap.add_argument("--only-served", action="store_true", help="only the served-requests measurement")
    ap.add_argument("--served-buffers", default="pinned", choices=["pinned", "pageable"],
                    help="host memory of the served requests' arrays and hit buffers (both paths)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import lbvh_gb300 as lb
    from lbvh_gb300 import _build

    _build.build()
    hbm_peak, peak_kind = peaks()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    ctx = lb.Context(local, stream.cuda_stream)
    from lbvh_gb300 import _lib

    if args.trace_refill is not None:
        ctx.set_param(_lib.PARAM_TRACE_REFILL, args.trace_refill)
    if args.trace_blocks is not None:
        ctx.set_param(_lib.PARAM_TRACE_BLOCKS_PER_SM, args.trace_blocks)
    if args.trace_leaf_batch is not None:
        ctx.set_param(_lib.PARAM_TRACE_LEAF_BATCH, args.trace_leaf_batch)
    if args.trace_ray_order is not None:
        ctx.set_param(_lib.PARAM_TRACE_RAY_ORDER, args.trace_ray_order)
    if args.tree_walk_fused is not None:
        ctx.set_param(_lib.PARAM_TREE_WALK_FUSED, args.tree_walk_fused)
    if args.small_build_max is not None:
        ctx.set_param(_lib.PARAM_SMALL_BUILD_MAX, args.small_build_max)

    def detail(name, rec):
        if rank == 0:
            print(json.dumps({"detail": name, name: rec}), flush=True)

    if args.only_served:
        detail("served", measure_served(local, buffers=args.served_buffers))
        return 0
    if args.only_batched:
        detail("batched", measure_batched(local, args.steps, hbm_peak, peak_kind))
        return 0
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)  # 256 MB > L2
    if args.only_config1:
        detail("config1", measure_config1(ctx, stream, flush, dev, args.steps))
        return 0
    if args.only_16m:
        detail("build_16m", measure_build_16m(ctx, lb.Builder(ctx), stream, flush, dev, args.steps, hbm_peak,
                                              peak_kind, args.soup_n, args.soup_span))
        return 0

    # ---- the step's inputs: the room, its primary rays, the bounce rays ---
    tris_h, prim_h = room_workload()
    if args.step_rays > 1:
        prim_h = np.ascontiguousarray(prim_h[:: args.step_rays])
    n = tris_h.shape[0]
    tris = torch.from_numpy(tris_h).to(dev)
    prim = torch.from_numpy(prim_h).to(dev)
    hits_p = torch.empty((prim.shape[0], 4), dtype=torch.float32, device=dev)
    builder = lb.Builder(ctx)
    bvh = lb.BVH(ctx)
    ctx.reserve(n, prim.shape[0])
    from lbvh_gb300 import autotune

    tuning = autotune.tune_build(ctx, tris)  # the room's size class: sort / bounds setting
    builder(tris, into=bvh)
    trav = lb.Traverser(bvh)
    trav(prim, out=hits_p)
    torch.cuda.synchronize()
    bounce_h = room_bounce(prim_h, lb.hits_view(hits_p), tris_h)  # made once, before timing
    bounce = torch.from_numpy(bounce_h).to(dev)
    hits_b = torch.empty((bounce.shape[0], 4), dtype=torch.float32, device=dev)
    m = prim.shape[0] + bounce.shape[0]
    config = room_config(tris_h, prim_h, bounce_h, world)
    # the traversal's leaf batching, refill, grid and ray order, tuned on the
    # step's own two traces (a sparse sample neither fills the GPU nor keeps
    # the rays' coherence)
    trace_tuning = dict(autotune.tune_trace(ctx, bvh, [prim, bounce], key=f"gb300:trace:{WORKLOAD}"))
    for flag, key in (("trace_refill", "trace_refill"), ("trace_blocks", "trace_blocks_per_sm"),
                      ("trace_leaf_batch", "trace_leaf_batch"), ("trace_ray_order", "trace_ray_order")):
        if getattr(args, flag) is not None:  # an explicit setting overrides the tuned one
            trace_tuning[key] = getattr(args, flag)
            autotune.apply(ctx, {key: trace_tuning[key]})

    for _ in range(args.warmup):
        builder(tris, into=bvh)
        trav(prim, out=hits_p)
        trav(bounce, out=hits_b)
    torch.cuda.synchronize()

    # ---- timed region: K whole steps --------------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.mark(True)
    t = time_steps(builder, bvh, trav, tris, [prim, bounce], [hits_p, hits_b], flush, stream, args.steps)
    clocks.mark(False)
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    build_ms = float(np.mean([x for x, _ in t]))
    trace_ms = float(np.mean([y for _, y in t]))
    step_ms, value = replica_throughput(build_ms + trace_ms, m, world, dev)
    gpu_launches = args.steps * step_launches(n, tuning, trace_tuning)

    # correctness guard on the timed output: the same hits as a fresh build
    ref_p = torch.empty_like(hits_p)
    ref_b = torch.empty_like(hits_b)
    fresh = lb.Traverser(lb.Builder(ctx)(tris))
    fresh(prim, out=ref_p)
    fresh(bounce, out=ref_b)
    torch.cuda.synchronize()
    assert torch.equal(ref_p.view(torch.int32), hits_p.view(torch.int32))
    assert torch.equal(ref_b.view(torch.int32), hits_b.view(torch.int32))
    hit_frac = float(np.mean(lb.hits_view(hits_p)["prim"] != lb.MISS))

    # ---- e2e: the public API with page-locked host buffers ---------------
    tris_pin = torch.from_numpy(tris_h).pin_memory()
    prim_pin = torch.from_numpy(prim_h).pin_memory()
    bounce_pin = torch.from_numpy(bounce_h).pin_memory()
    out_p = torch.empty((prim.shape[0], 4), dtype=torch.float32).pin_memory()
    out_b = torch.empty((bounce.shape[0], 4), dtype=torch.float32).pin_memory()
    if args.e2e_chunk is not None:
        ctx.set_param(_lib.PARAM_TRACE_CHUNK, args.e2e_chunk)
    b_e2e = lb.BVH(ctx)
    builder(tris_pin, into=b_e2e)
    # how the host rays and hits travel (in place over the CPU-GPU link, or
    # copied), tuned on these very buffers
    transfer = autotune.tune_transfer(ctx, b_e2e, [(prim_pin, out_p), (bounce_pin, out_b)],
                                      key=f"gb300:transfer:{WORKLOAD}")
    if args.e2e_in_place is not None:
        ctx.set_param(_lib.PARAM_TRACE_IN_PLACE, args.e2e_in_place)
    for _ in range(2):
        tr = lb.Traverser(builder(tris_pin, into=b_e2e))
        tr(prim_pin, out=out_p)
        tr(bounce_pin, out=out_b)
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        builder(tris_pin, into=b_e2e)        # H2D copy of the triangles inside
        tr = lb.Traverser(b_e2e)
        tr(prim_pin, out=out_p)              # rays read / hits written in host memory, synchronous
        tr(bounce_pin, out=out_b)
        e2e_t.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * float(np.mean(e2e_t))
    assert torch.equal(out_p.view(torch.int32), hits_p.cpu().view(torch.int32))
    assert torch.equal(out_b.view(torch.int32), hits_b.cpu().view(torch.int32))
    del tris_pin, prim_pin, bounce_pin, out_p, out_b

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config,
        "build": {"ms": round(build_ms, 4), "mprims_s": round(n / (build_ms * 1e-3) / 1e6, 1),
                  "tuning": {k: tuning[k] for k in ("sort_tile_keys", "bucket_sort_min", "bounds_blocks_per_sm")}},
        "trace": {"ms": round(trace_ms, 4), "mrays_s": round(m / (trace_ms * 1e-3) / 1e6, 1),
                  "primary_hit_fraction": round(hit_frac, 4),
                  "tuning": {k: trace_tuning.get(k, 0) for k in ("trace_leaf_batch", "trace_refill", "trace_blocks_per_sm",
                                                                  "trace_ray_order")}},
    }
    detail("build_tuning", tuning)
    detail("trace_tuning", trace_tuning)
    line["e2e"] = {"value": round(world * m / (e2e_ms * 1e-3) / 1e6, 3), "unit": "Mrays/s",
                   "ms_per_step": round(e2e_ms, 4), "trace_in_place": int(ctx_in_place(ctx, transfer, args))}
    detail("transfer_tuning", transfer)
    if args.only_step:
        line["gpu_launches"] = gpu_launches
        line["clocks"] = clk
        if rank == 0:
            print(json.dumps(line), flush=True)
        return 0

    # ---- the mid-size torus step -------------------------------------------
    if not args.no_config1:
        line["config1"] = measure_config1(ctx, stream, flush, dev, args.steps)
        detail("config1", line["config1"])

    # ---- served requests vs the plain path (before the large workloads) ---
    if not args.no_served:
        line["served"] = measure_served(local, buffers=args.served_buffers)
        detail("served", line["served"])

    # ---- 16M-triangle build: the HBM roofline workload ---------------------
    if not args.no_16m:
        line["build_16m"] = measure_build_16m(ctx, builder, stream, flush, dev, args.steps, hbm_peak, peak_kind,
                                              args.soup_n, with_refit=True)
        detail("build_16m", line["build_16m"])

    # ---- batched meshes (4,096 soups) vs the plain per-mesh path ----------
    if not args.no_batched:
        line["batched"] = measure_batched(local, args.steps, hbm_peak, peak_kind)
        detail("batched", line["batched"])

    # ---- roofline: the build (HBM-bound) at 16M triangles, or the step's
    # own build when that measurement was skipped; the traversal (issue /
    # latency bound) is described by its ncu figures beside it
    if line.get("build_16m"):
        rf = dict(line["build_16m"]["roofline"], kernel="lbvh build, 16M-triangle soup (all build kernels)")
    else:
        algo = n * sum(BYTES_PER_PRIM.values())
        rf = {"bound": "hbm", "kernel": "lbvh build, room scene (all build kernels)",
              "achieved": round(algo / (build_ms * 1e-3) / 1e9, 1), "peak": hbm_peak, "unit": "GB/s",
              "frac": round(algo / (build_ms * 1e-3) / 1e9 / hbm_peak, 4),
              "bytes_per_prim": sum(BYTES_PER_PRIM.values()), "traffic": None, "peak_kind": peak_kind}
    line["roofline"] = rf
    line["trace_profile"] = measured_profile("k_trace_room", ("issue_slots_busy", "simt_threads_per_instruction",
                                                              "l1_hit_rate", "l2_hit_rate", "warps_active_of_max"))

    # ---- CPU baseline: the reference on the host cores (bounded sample) ---
    if rank == 0 and not args.no_cpu:
        impl, kind, path = cpu_impl()
        cores = os.cpu_count() or 1
        sp, sb = np.ascontiguousarray(prim_h[::16]), np.ascontiguousarray(bounce_h[::16])
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            nodes = impl.build(tris_h, cores)
            impl.trace(nodes, tris_h, sp, cores)
            impl.trace(nodes, tris_h, sb, cores)
            ts.append(time.perf_counter() - t0)
        cval = (sp.shape[0] + sb.shape[0]) / float(np.mean(ts)) / 1e6
        line["cpu_baseline"] = {"value": round(cval, 4), "unit": "Mrays/s", "cores": cores, "kind": kind,
                                "lib": os.path.relpath(path, ROOT),
                                "sample": f"build of all {n} triangles + every 16th primary and bounce ray "
                                          f"({sp.shape[0] + sb.shape[0]}) per step, 3 steps"}
    line["e2e"] = {"value": round(world * m / (e2e_ms * 1e-3) / 1e6, 3), "unit": "Mrays/s",
                   "ms_per_step": round(e2e_ms, 4),
                   "h2d_bytes_per_step": int(tris_h.nbytes + prim_h.nbytes + bounce_h.nbytes),
                   "d2h_bytes_per_step": int(m * 16),
                   "trace_in_place": line["e2e"]["trace_in_place"],
                   "transfer": TRANSFER_NOTE[line["e2e"]["trace_in_place"]]}
    line["gpu_launches"] = gpu_launches
    line["clocks"] = clk
    if rank == 0:
        print(json.dumps(summary_line(line)), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
