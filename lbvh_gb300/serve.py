"""Request server: build / refit / trace requests on device-resident BVHs.

`Server` is the Python face of the native server in the shared library
(lbvh_server_*, lbvh_gb300/csrc/server.cu). Requests arrive over time
(submit() from any thread returns a Future); inside the library one dispatch
thread decides what runs and `slots` worker threads, each with its own CUDA
stream and lbvh context, run it, so work admitted while other work is on the
GPU runs concurrently with it (continuous batching, not a queue drained one
request at a time):

* every scene's BVH stays resident on the device between requests;
* admission is against an HBM budget: a request that needs memory evicts
  least-recently-used resident scenes that no queued or running request
  needs, and otherwise waits until running work frees memory; an evicted
  scene's tree is dumped to host memory (within `host_budget`) and loaded
  back, checked, by its next trace or refit;
* small builds (at most `batch_max_tris` triangles) waiting together are
  coalesced into one batched build (lbvh_batch_build_triangles); small
  traces queued together against one tree become one trace launch, and those
  against scenes of the same batch one batched trace;
* requests on one scene keep their submission order (a trace submitted after
  a refit sees the refitted tree); requests on different scenes overlap.
  Waiting requests sit in one queue per scene, so choosing the next job
  costs time in the number of scenes, not of waiting requests.

Host data moves straight between the caller's (pageable) arrays and the
device, each request's copy issued by the worker that runs it: on a
Grace-Blackwell node the copy engines read and write pageable memory through
the shared address space at full link speed, while a CPU copy into a pinned
staging buffer runs at single-core memcpy speed, so no staging buffers are
used. No Python runs between a request's arrival and its completion except
submit() and the thread that resolves the futures.

Every result equals running the same request alone through the plain API
(Builder / BVH.refit / Traverser): the kernels are the same and the
arithmetic is bit-identical to the reference.

Latency = completion of the request's GPU work and result copy, as seen by
the worker that ran it, minus arrival (submit) time, both on the server's
clock.

Failures stay on the host and leave the server serving: a request cancelled
before it started (`cancel`) raises CancelledError, one still queued
`max_queue_s` after its arrival raises TimeoutError, a device allocation that
fails raises MemoryError (a rebuild that fails keeps the scene's previous
tree), and `inject_alloc_failures` makes the next allocations fail on purpose
so that tests can exercise that path.
"""
from __future__ import annotations

import ctypes
import threading
import time
from concurrent.futures import CancelledError, Future
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from . import api as lbapi

BUILD, REFIT, TRACE = "build", "refit", "trace"
_KINDS = {BUILD: _lib.REQ_BUILD, REFIT: _lib.REQ_REFIT, TRACE: _lib.REQ_TRACE}


@dataclass(eq=False)  # requests are compared by identity
class Request:
    kind: str
    scene: int
    data: np.ndarray  # triangles [n, 12] (build, refit) or rays [m, 8] (trace)
    result: object = None   # trace: the HIT_DTYPE array the hits land in
    arrival: float = 0.0    # seconds on the server's clock
    started: float = 0.0
    done: float = 0.0
    future: Future = field(default_factory=Future)


def scene_bytes(n: int) -> int:
    """Device bytes a resident scene of n triangles holds: triangles (48),
    nodes (32), traversal copy (64), sorted codes (4) per triangle."""
    return 148 * n + (1 << 16)


def _exception(status: int, msg: str) -> BaseException:
    if status == _lib.LBVH_ERR_NOT_RESIDENT:
        return KeyError(msg)
    if status == _lib.LBVH_ERR_INVALID_ARG:
        return ValueError(msg)
    if status in (_lib.LBVH_ERR_BUDGET, _lib.LBVH_ERR_OOM):
        return MemoryError(msg)
    if status == _lib.LBVH_ERR_CANCELLED:
        return CancelledError(msg)
    if status == _lib.LBVH_ERR_EXPIRED:
        return TimeoutError(msg)
    return _lib.LbvhError(status, msg)


class Server:
    """See the module docstring. Results: build / refit -> None,
    trace -> HIT_DTYPE array."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int = 120 << 30,
                 batch_max_tris: int = 65536, batch_max_requests: int = 128,
                 trace_batch_max_rays: int = 1 << 16, host_budget: int = 64 << 30, max_queue_s: float = 0.0):
        L = _lib.lib()
        cfg = _lib.ServerConfig(int(device), int(slots), int(hbm_budget), int(batch_max_tris),
                                int(batch_max_requests), int(trace_batch_max_rays), int(host_budget),
                                float(max_queue_s))
        h = ctypes.c_void_p()
        st = L.lbvh_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if st:
            raise _exception(st, f"server creation failed ({_lib.status_string(st)})")
        self._h = h
        self.device = device
        self.budget = int(hbm_budget)
        self.done: list[Request] = []
        self._waiting: dict[int, Request] = {}
        self._lock = threading.Lock()
        self._closing = False
        self._collector = threading.Thread(target=self._collect, name="lbvh-server-results", daemon=True)
        self._collector.start()

    # ---- public --------------------------------------------------------------
    def submit(self, kind: str, scene: int, data, out: np.ndarray | None = None) -> Future:
        """Queues a request; a trace's hits go to `out` (rows HIT_DTYPE
        records, e.g. a buffer the caller reuses) or to a new array."""
        if kind not in _KINDS:
            raise ValueError(f"unknown request kind {kind!r}")
        width = 8 if kind == TRACE else 12
        data = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, width)
        rows = data.shape[0]
        hits = None
        if kind == TRACE:
            hits = np.empty(rows, lbapi.HIT_DTYPE) if out is None else out
            if hits.dtype != lbapi.HIT_DTYPE or hits.shape != (rows,) or not hits.flags.c_contiguous:
                raise ValueError(f"out must be a contiguous array of {rows} HIT_DTYPE records")
        r = Request(kind, int(scene), data, result=hits)
        ticket = ctypes.c_uint64()
        with self._lock:
            if self._closing:
                raise RuntimeError("server is closed")
            st = _lib.lib().lbvh_server_submit(self._h, _KINDS[kind], int(scene), data.ctypes.data, rows,
                                               None if hits is None else hits.ctypes.data, ctypes.byref(ticket))
            if st:
                raise _exception(st, "request rejected")
            self._waiting[ticket.value] = r  # keeps data and hits alive until done
        r.future.ticket = ticket.value
        return r.future

    def cancel(self, future: Future) -> None:
        """Cancels the request behind `future` if it has not started (its
        result then raises CancelledError); a started request finishes."""
        _lib.lib().lbvh_server_cancel(self._h, future.ticket)

    def inject_alloc_failures(self, count: int) -> None:
        """Test hook: the next `count` device allocations of the server's
        workers fail as on an exhausted device (those requests raise
        MemoryError)."""
        _lib.lib().lbvh_server_inject_alloc_failures(self._h, int(count))

    def close(self, wait: bool = True) -> None:
        """Finishes every submitted request, then frees the server."""
        if self._h is None:
            return
        with self._lock:
            self._closing = True
        _lib.lib().lbvh_server_drain(self._h)
        self._collector.join()
        _lib.lib().lbvh_server_destroy(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def clock(self) -> float:
        """The server's clock (seconds), on which Request times are given."""
        return float(_lib.lib().lbvh_server_clock(self._h))

    def _stats(self) -> _lib.ServerStats:
        out = _lib.ServerStats()
        _lib.lib().lbvh_server_stats_get(self._h, ctypes.byref(out))
        return out

    @property
    def coalesced(self) -> int:
        return int(self._stats().coalesced_requests)

    @property
    def evictions(self) -> int:
        return int(self._stats().evictions)

    @property
    def spills(self) -> int:
        """Evicted scenes dumped to host memory."""
        return int(self._stats().spills)

    @property
    def reloads(self) -> int:
        """Dumped scenes loaded back onto the device."""
        return int(self._stats().reloads)

    @property
    def spilled(self) -> int:
        return int(self._stats().spilled_scenes)

    @property
    def cancelled(self) -> int:
        return int(self._stats().cancelled)

    @property
    def expired(self) -> int:
        return int(self._stats().expired)

    @property
    def used(self) -> int:
        return int(self._stats().resident_bytes)

    @property
    def resident(self) -> list[int]:
        n = ctypes.c_size_t()
        L = _lib.lib()
        L.lbvh_server_resident(self._h, None, 0, ctypes.byref(n))
        buf = (ctypes.c_int64 * max(1, n.value))()
        L.lbvh_server_resident(self._h, buf, n.value, ctypes.byref(n))
        return [int(buf[k]) for k in range(min(n.value, len(buf)))]

    # ---- results -----------------------------------------------------------------
    def _collect(self):
        L = _lib.lib()
        cap = 256
        buf = (_lib.RequestDone * cap)()
        n = ctypes.c_size_t()
        while True:
            L.lbvh_server_wait_any(self._h, buf, cap, 0.05, ctypes.byref(n))
            for k in range(n.value):
                d = buf[k]
                with self._lock:
                    r = self._waiting.pop(d.ticket)
                r.arrival, r.started, r.done = d.arrival, d.start, d.done
                self.done.append(r)
                if d.status == _lib.LBVH_OK:
                    r.future.set_result(r.result)
                else:
                    r.future.set_exception(_exception(d.status, d.message.decode(errors="replace")))
            with self._lock:
                if self._closing and not self._waiting:
                    return


def run_plain(requests, device: int = 0, outs=None):
    """The same requests through the plain API, one at a time in arrival
    order on one stream, each starting no earlier than its arrival time
    (seconds after the start). A trace writes its hits to outs[i] when given.
    Returns [(result, latency_s)]."""
    import torch

    ctx = lbapi.Context(device, torch.cuda.current_stream(device).cuda_stream)
    scenes = {}
    out = []
    t0 = time.perf_counter()
    for i, (at, kind, scene, data) in enumerate(requests):
        now = time.perf_counter() - t0
        if now < at:
            time.sleep(at - now)
        arrival = t0 + at
        if kind == BUILD:
            tris = torch.from_numpy(np.ascontiguousarray(data)).to(device)
            scenes[scene] = (lbapi.Builder(ctx)(tris), tris)
            torch.cuda.synchronize()
            res = None
        elif kind == REFIT:
            tris = torch.from_numpy(np.ascontiguousarray(data)).to(device)
            bvh, _ = scenes[scene]
            bvh.refit(tris)
            scenes[scene] = (bvh, tris)
            torch.cuda.synchronize()
            res = None
        else:
            res = lbapi.Traverser(scenes[scene][0])(np.ascontiguousarray(data), out=None if outs is None else outs[i])
        out.append((res, time.perf_counter() - arrival))
    return out
