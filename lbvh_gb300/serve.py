"""Request server: build / refit / trace requests on device-resident BVHs.

Requests arrive over time (submit() from any thread) and are served by one
dispatch thread over `slots` CUDA streams, each with its own lbvh context, so
work admitted while other work is on the GPU runs concurrently with it
(continuous batching, not a queue drained one request at a time):

* every scene's BVH stays resident on the device between requests;
* admission is against an HBM budget: a request that needs memory evicts
  least-recently-used resident scenes that no queued or running request
  needs, and otherwise waits until running work frees memory;
* small builds (at most `batch_max_tris` triangles) waiting together are
  coalesced into one batched build (lbvh_batch_build_triangles), and small
  traces against scenes of the same batch into one batched trace;
* requests on one scene keep their submission order (a trace submitted after
  a refit sees the refitted tree); requests on different scenes overlap.

Every result equals running the same request alone through the plain API
(Builder / BVH.refit / Traverser): the kernels are the same and the
arithmetic is bit-identical to the reference.

Latency = completion seen by the dispatcher - arrival (submit) time.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import api as lbapi

BUILD, REFIT, TRACE = "build", "refit", "trace"


@dataclass(eq=False)  # requests are compared by identity
class Request:
    kind: str
    scene: int
    data: np.ndarray  # triangles [n, 12] (build, refit) or rays [m, 8] (trace)
    arrival: float = 0.0
    future: Future = field(default_factory=Future)
    started: float = 0.0
    done: float = 0.0


@dataclass(eq=False)
class Resident:
    """A scene on the device: its own BVH, or member `index` of a batch."""
    n: int
    nbytes: int
    bvh: object = None          # lbapi.BVH
    tris: object = None         # device triangles the BVH borrows
    batch: object = None        # _BatchRef
    index: int = -1
    busy: int = 0               # running requests that read it
    last_use: float = 0.0
    retired: bool = False       # replaced or evicted, freed when busy drops to 0


@dataclass(eq=False)
class _BatchRef:
    batch: object               # lbapi.Batch
    tris: object                # device triangles of all members
    offsets: np.ndarray         # host copy of the member offsets
    members: int = 0            # members still resident


def scene_bytes(n: int) -> int:
    """Device bytes a resident scene of n triangles holds: triangles (48),
    nodes (32), traversal copy (64) per triangle."""
    return 144 * n + (1 << 16)


class _Slot:
    def __init__(self, torch, device: int):
        self.stream = torch.cuda.Stream(device)
        self.ctx = lbapi.Context(device, self.stream.cuda_stream)
        self.busy = False
        self.pinned = {}

    def pinned_buffer(self, torch, key: str, nbytes: int):
        buf = self.pinned.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8).pin_memory()
            self.pinned[key] = buf
        return buf[:nbytes]


class Server:
    """See the module docstring. Results: build / refit -> None,
    trace -> HIT_DTYPE array."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int = 120 << 30,
                 batch_max_tris: int = 65536, batch_max_requests: int = 128,
                 trace_batch_max_rays: int = 1 << 16):
        import torch

        self.torch = torch
        self.device = device
        self.slots = [_Slot(torch, device) for _ in range(slots)]
        self.budget = int(hbm_budget)
        self.used = 0
        self.batch_max_tris = batch_max_tris
        self.batch_max_requests = batch_max_requests
        self.trace_batch_max_rays = trace_batch_max_rays
        self.resident: "collections.OrderedDict[int, Resident]" = collections.OrderedDict()
        self.writing: set[int] = set()        # scenes with a running build / refit
        self.pending: collections.deque[Request] = collections.deque()
        self.running: list = []               # (event, slot, finish callback)
        self.done: list[Request] = []
        self.evictions = 0
        self.coalesced = 0
        self._cv = threading.Condition()
        self._stop = False
        self._error = None
        self._thread = threading.Thread(target=self._loop, name="lbvh-server", daemon=True)
        self._thread.start()

    # ---- public --------------------------------------------------------------
    def submit(self, kind: str, scene: int, data: np.ndarray) -> Future:
        if kind not in (BUILD, REFIT, TRACE):
            raise ValueError(f"unknown request kind {kind!r}")
        width = 8 if kind == TRACE else 12
        data = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, width)
        r = Request(kind, int(scene), data, arrival=time.perf_counter())
        with self._cv:
            if self._stop:
                raise RuntimeError("server is closed")
            self.pending.append(r)
            self._cv.notify()
        return r.future

    def close(self, wait: bool = True) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify()
        if wait:
            self._thread.join()
        if self._error is not None:
            raise self._error

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- dispatch loop ---------------------------------------------------------
    def _loop(self):
        try:
            while True:
                with self._cv:
                    if self._stop and not self.pending and not self.running:
                        return
                progressed = self._poll()
                progressed |= self._dispatch()
                if not progressed:
                    with self._cv:
                        if not self._stop or self.pending or self.running:
                            self._cv.wait(timeout=2e-5 if self.running else 1e-3)
        except BaseException as exc:  # fail every waiting request, keep the cause
            self._error = exc
            with self._cv:
                rest = list(self.pending)
                self.pending.clear()
            for r in rest:
                if not r.future.done():
                    r.future.set_exception(exc)

    def _poll(self) -> bool:
        progressed = False
        still = []
        for ev, slot, finish in self.running:
            if ev.query():
                finish()
                slot.busy = False
                progressed = True
            else:
                still.append((ev, slot, finish))
        self.running = still
        return progressed

    def _pending_scenes(self, exclude=()) -> set[int]:
        with self._cv:
            return {r.scene for r in self.pending if r not in exclude}

    def _admissible(self, r: Request) -> bool:
        res = self.resident.get(r.scene)
        if r.scene in self.writing:
            return False
        if r.kind == TRACE:
            return res is not None
        if r.kind == REFIT:
            return res is not None and res.busy == 0 and res.n == r.data.shape[0]
        return self._make_room(scene_bytes(r.data.shape[0]), keep={r.scene})

    def _make_room(self, need: int, keep: set[int]) -> bool:
        if self.used + need <= self.budget:
            return True
        wanted = self._pending_scenes() | keep
        for scene in list(self.resident):
            if self.used + need <= self.budget:
                break
            res = self.resident[scene]
            if res.busy or scene in wanted or scene in self.writing:
                continue
            self._drop(scene)
            self.evictions += 1
        return self.used + need <= self.budget

    def _drop(self, scene: int) -> None:
        """Takes a scene out of residency; its memory goes back once no
        running request reads it."""
        res = self.resident.pop(scene, None)
        if res is None:
            return
        res.retired = True
        if res.busy == 0:
            self._release(res)

    def _release(self, res: Resident) -> None:
        self.used -= res.nbytes
        if res.batch is not None:
            res.batch.members -= 1
            if res.batch.members == 0:
                res.batch.batch.close()
        elif res.bvh is not None:
            res.bvh.close()

    def _dispatch(self) -> bool:
        free = [s for s in self.slots if not s.busy]
        if not free:
            return False
        with self._cv:
            queue = list(self.pending)
        if not queue:
            return False
        blocked: set[int] = set()
        builds_ahead: set[int] = set()
        chosen = None
        for r in queue:
            if r.scene in blocked:
                continue
            if r.kind != BUILD and r.scene not in self.resident and r.scene not in self.writing \
                    and r.scene not in builds_ahead:
                self._take([r])
                r.future.set_exception(KeyError(f"scene {r.scene} is not resident"))
                return True
            if self._admissible(r):
                chosen = r
                break
            blocked.add(r.scene)
            if r.kind == BUILD:
                builds_ahead.add(r.scene)
        if chosen is None:
            return False
        slot = free[0]
        if chosen.kind == BUILD:
            group = [chosen]
            if chosen.data.shape[0] <= self.batch_max_tris:
                seen = {chosen.scene}
                for r in queue:
                    if len(group) >= self.batch_max_requests:
                        break
                    if r is chosen or r.kind != BUILD or r.scene in seen or r.scene in blocked:
                        seen.add(r.scene)
                        continue
                    seen.add(r.scene)
                    if r.data.shape[0] <= self.batch_max_tris and self._admissible(r):
                        group.append(r)
            self._take(group)
            if len(group) > 1:
                self.coalesced += len(group)
                self._start_batch_build(slot, group)
            else:
                self._start_build(slot, chosen)
        elif chosen.kind == REFIT:
            self._take([chosen])
            self._start_refit(slot, chosen)
        else:
            res = self.resident[chosen.scene]
            group = [chosen]
            if res.batch is not None and chosen.data.shape[0] <= self.trace_batch_max_rays:
                # a trace may run ahead of other traces, never ahead of an
                # earlier build or refit of its scene
                stopped = set(blocked)
                for r in queue:
                    if r is chosen:
                        continue
                    if r.kind != TRACE:
                        stopped.add(r.scene)
                        continue
                    if r.scene in stopped:
                        continue
                    other = self.resident.get(r.scene)
                    if other is not None and other.batch is res.batch and r.scene not in self.writing \
                            and r.data.shape[0] <= self.trace_batch_max_rays:
                        group.append(r)
            self._take(group)
            if len(group) > 1:
                self.coalesced += len(group)
            self._start_trace(slot, group)
        return True

    def _take(self, group) -> None:
        now = time.perf_counter()
        with self._cv:
            for r in group:
                self.pending.remove(r)
                r.started = now

    def _finish(self, group, results=None) -> None:
        now = time.perf_counter()
        for k, r in enumerate(group):
            r.done = now
            self.done.append(r)
            r.future.set_result(None if results is None else results[k])

    def _launch(self, slot, finish) -> None:
        ev = self.torch.cuda.Event()
        ev.record(slot.stream)
        slot.busy = True
        self.running.append((ev, slot, finish))

    def _upload(self, slot, key: str, host: np.ndarray):
        """Host array -> new device tensor, through the slot's pinned buffer,
        on the slot's stream."""
        torch = self.torch
        nbytes = host.nbytes
        pin = slot.pinned_buffer(torch, key, nbytes)
        pin.numpy()[:nbytes] = host.reshape(-1).view(np.uint8)
        with torch.cuda.stream(slot.stream):
            dev = torch.empty(host.shape, dtype=torch.float32, device=self.device)
            dev.view(torch.uint8).view(-1).copy_(pin, non_blocking=True)
        return dev

    def _check(self, slot, status: int) -> None:
        slot.ctx.check(status)

    # ---- jobs ------------------------------------------------------------------
    def _start_build(self, slot, r: Request) -> None:
        from . import _lib

        n = r.data.shape[0]
        self.used += scene_bytes(n)
        self.writing.add(r.scene)
        dev = self._upload(slot, "tris", r.data)
        bvh = lbapi.BVH(slot.ctx)
        self._check(slot, _lib.lib().lbvh_build_triangles(slot.ctx.handle, dev.data_ptr(), n, 0, bvh.handle))
        # the traversal copy is made here, on this stream, so that traces on
        # other streams never build it concurrently
        self._check(slot, _lib.lib().lbvh_bvh_prepare_trace(slot.ctx.handle, bvh.handle))
        bvh.kind = lbapi.TRIANGLES

        def finish():
            self._drop(r.scene)
            self.resident[r.scene] = Resident(n, scene_bytes(n), bvh=bvh, tris=dev, last_use=time.perf_counter())
            self.writing.discard(r.scene)
            self._finish([r])

        self._launch(slot, finish)

    def _start_batch_build(self, slot, group) -> None:
        from . import _lib

        counts = np.array([r.data.shape[0] for r in group], np.int64)
        offsets = np.zeros(len(group) + 1, np.uint32)
        offsets[1:] = np.cumsum(counts)
        for r in group:
            self.used += scene_bytes(r.data.shape[0])
            self.writing.add(r.scene)
        dev = self._upload(slot, "tris", np.concatenate([r.data for r in group]))
        batch = lbapi.Batch(slot.ctx)
        self._check(slot, _lib.lib().lbvh_batch_build_triangles(slot.ctx.handle, dev.data_ptr(), int(offsets[-1]),
                                                               offsets.ctypes.data, len(group), batch._h))
        self._check(slot, _lib.lib().lbvh_batch_prepare_trace(slot.ctx.handle, batch._h))
        batch._keep = (dev, offsets)
        batch._offsets = offsets
        ref = _BatchRef(batch, dev, offsets, members=len(group))

        def finish():
            now = time.perf_counter()
            for k, r in enumerate(group):
                self._drop(r.scene)
                n = r.data.shape[0]
                self.resident[r.scene] = Resident(n, scene_bytes(n), batch=ref, index=k, last_use=now)
                self.writing.discard(r.scene)
            self._finish(group)

        self._launch(slot, finish)

    def _standalone(self, slot, scene: int) -> Resident:
        """Moves a batch member into its own BVH (same nodes), for a refit."""
        res = self.resident[scene]
        ref, k = res.batch, res.index
        o = ref.offsets
        nodes = ref.batch.mesh_nodes(k)
        tris = ref.tris[int(o[k]) : int(o[k + 1])]
        bvh = lbapi.BVH.from_nodes(nodes, tris, slot.ctx)
        res.retired = True  # the batch member leaves; its traces have finished (refits need busy == 0)
        ref.members -= 1
        if ref.members == 0:
            ref.batch.close()
        new = Resident(res.n, res.nbytes, bvh=bvh, tris=tris, busy=res.busy, last_use=res.last_use)
        self.resident[scene] = new
        return new

    def _start_refit(self, slot, r: Request) -> None:
        from . import _lib

        res = self.resident[r.scene]
        if res.batch is not None:
            res = self._standalone(slot, r.scene)
        self.writing.add(r.scene)
        dev = self._upload(slot, "tris", r.data)
        self._check(slot, _lib.lib().lbvh_refit_triangles(slot.ctx.handle, res.bvh.handle, dev.data_ptr()))
        self._check(slot, _lib.lib().lbvh_bvh_prepare_trace(slot.ctx.handle, res.bvh.handle))

        def finish():
            res.tris = dev  # the refitted BVH now borrows these triangles
            res.last_use = time.perf_counter()
            self.resident.move_to_end(r.scene)
            self.writing.discard(r.scene)
            self._finish([r])

        self._launch(slot, finish)

    def _start_trace(self, slot, group) -> None:
        from . import _lib

        torch = self.torch
        res0 = self.resident[group[0].scene]
        used = [self.resident[r.scene] for r in group]
        for res in used:
            res.busy += 1
        if res0.batch is None:
            r = group[0]
            m = r.data.shape[0]
            rays = self._upload(slot, "rays", r.data)
            with torch.cuda.stream(slot.stream):
                hits = torch.empty((m, 4), dtype=torch.float32, device=self.device)
            self._check(slot, _lib.lib().lbvh_trace_triangles(slot.ctx.handle, res0.bvh.handle, rays.data_ptr(), m,
                                                             hits.data_ptr()))
            spans = [(0, m)]
        else:
            ref = res0.batch
            nm = ref.offsets.size - 1
            order = sorted(range(len(group)), key=lambda k: self.resident[group[k].scene].index)
            per_mesh = np.zeros(nm, np.int64)
            for k in order:
                per_mesh[self.resident[group[k].scene].index] += group[k].data.shape[0]
            roff = np.zeros(nm + 1, np.uint32)
            roff[1:] = np.cumsum(per_mesh)
            cursor = roff[:-1].astype(np.int64).copy()
            spans = [None] * len(group)
            chunks = [None] * len(group)
            for k in order:
                idx = self.resident[group[k].scene].index
                m_k = group[k].data.shape[0]
                spans[k] = (int(cursor[idx]), int(cursor[idx]) + m_k)
                cursor[idx] += m_k
            allr = np.empty((int(roff[-1]), 8), np.float32)
            for k, r in enumerate(group):
                allr[spans[k][0] : spans[k][1]] = r.data
            m = allr.shape[0]
            rays = self._upload(slot, "rays", allr)
            with torch.cuda.stream(slot.stream):
                hits = torch.empty((m, 4), dtype=torch.float32, device=self.device)
            self._check(slot, _lib.lib().lbvh_batch_trace_triangles(slot.ctx.handle, ref.batch._h, rays.data_ptr(),
                                                                   roff.ctypes.data, m, hits.data_ptr()))
        pin = slot.pinned_buffer(torch, "hits", 16 * m)
        with torch.cuda.stream(slot.stream):
            pin.copy_(hits.view(torch.uint8).view(-1), non_blocking=True)

        def finish():
            _ = (rays, hits)  # keep the device buffers alive until the GPU is done
            all_hits = pin.numpy().view(lbapi.HIT_DTYPE)
            results = [np.array(all_hits[a:b]) for a, b in spans]
            now = time.perf_counter()
            for r, res in zip(group, used):
                res.busy -= 1
                res.last_use = now
                if res.retired:
                    if res.busy == 0:
                        self._release(res)
                elif r.scene in self.resident:
                    self.resident.move_to_end(r.scene)
            self._finish(group, results)

        self._launch(slot, finish)


def run_plain(requests, device: int = 0):
    """The same requests through the plain API, one at a time in arrival
    order on one stream, each starting no earlier than its arrival time
    (seconds after the start). Returns [(result, latency_s)]."""
    import torch

    ctx = lbapi.Context(device, torch.cuda.current_stream(device).cuda_stream)
    scenes = {}
    out = []
    t0 = time.perf_counter()
    for at, kind, scene, data in requests:
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
            res = lbapi.Traverser(scenes[scene][0])(np.ascontiguousarray(data))
        out.append((res, time.perf_counter() - arrival))
    return out
