"""Request server: build / refit / trace requests on device-resident BVHs.

Requests arrive over time (submit() from any thread). One dispatch thread
decides what runs; `slots` worker threads, each with its own CUDA stream and
lbvh context, run it, so work admitted while other work is on the GPU runs
concurrently with it (continuous batching, not a queue drained one request
at a time):

* every scene's BVH stays resident on the device between requests;
* admission is against an HBM budget: a request that needs memory evicts
  least-recently-used resident scenes that no queued or running request
  needs, and otherwise waits until running work frees memory;
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
used. Result arrays are touched (one byte per page) while the kernel runs,
so the device-to-host copy lands in mapped pages.

Every result equals running the same request alone through the plain API
(Builder / BVH.refit / Traverser): the kernels are the same and the
arithmetic is bit-identical to the reference.

Latency = completion of the request's GPU work and result copy, as seen by
its worker, minus arrival (submit) time.
"""
from __future__ import annotations

import collections
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import _lib
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
    seq: int = 0


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


def _touch(a: np.ndarray) -> None:
    """Maps a fresh array's pages (one write per 4 KiB)."""
    b = a.reshape(-1).view(np.uint8)
    b[::4096] = 0


class _Job:
    __slots__ = ("work", "finish", "fail", "out", "err", "t_done")

    def __init__(self, work, finish, fail):
        self.work, self.finish, self.fail = work, finish, fail
        self.out = self.err = None
        self.t_done = 0.0


class _Slot:
    """A worker thread with its own stream and lbvh context. It runs one job
    at a time: the job's work() issues copies and launches on the stream,
    then the worker waits for the stream (and reads the context's device
    error word) before reporting the job complete to the dispatcher."""

    def __init__(self, server, torch, device: int, k: int):
        self.server = server
        self.torch = torch
        self.device = device
        self.stream = torch.cuda.Stream(device)
        self.ctx = lbapi.Context(device, self.stream.cuda_stream)
        self.busy = False
        self.jobs: queue.SimpleQueue = queue.SimpleQueue()
        self.thread = threading.Thread(target=self._run, name=f"lbvh-server-slot{k}", daemon=True)
        self.thread.start()

    def _run(self):
        torch = self.torch
        torch.cuda.set_device(self.device)
        while True:
            job = self.jobs.get()
            if job is None:
                return
            try:
                with torch.cuda.stream(self.stream):
                    job.out = job.work()
                self.ctx.synchronize()
            except BaseException as exc:  # reported to the job's requests
                job.err = exc
                try:
                    self.stream.synchronize()
                except BaseException:
                    pass
            job.t_done = time.perf_counter()
            self.server._completed(self, job)

    def upload(self, host: np.ndarray, width: int):
        """Host rows -> new device float32 tensor [rows, width] (allocated on
        this stream, copied straight from the host array)."""
        torch = self.torch
        dev = torch.empty((host.shape[0], width), dtype=torch.float32, device=self.device)
        dev.copy_(torch.from_numpy(host), non_blocking=True)
        return dev


class Server:
    """See the module docstring. Results: build / refit -> None,
    trace -> HIT_DTYPE array."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int = 120 << 30,
                 batch_max_tris: int = 65536, batch_max_requests: int = 128,
                 trace_batch_max_rays: int = 1 << 16):
        import torch

        self.torch = torch
        self.device = device
        self.budget = int(hbm_budget)
        self.used = 0
        self.batch_max_tris = batch_max_tris
        self.batch_max_requests = batch_max_requests
        self.trace_batch_max_rays = trace_batch_max_rays
        self.resident: "collections.OrderedDict[int, Resident]" = collections.OrderedDict()
        self.writing: set[int] = set()        # scenes with a running build / refit
        self._inbox: list[Request] = []       # submitted, not yet queued (guarded by _cv)
        self._seq = 0                         # submission counter (guarded by _cv)
        # waiting requests, one FIFO per scene (dispatch thread only): a
        # dispatch looks at the scenes' oldest requests, so its cost grows
        # with the number of scenes, not with the number of waiting requests
        self.queues: dict[int, collections.deque[Request]] = {}
        self.done: list[Request] = []
        self.evictions = 0
        self.coalesced = 0
        self._cv = threading.Condition()
        self._dirty = False                   # a submit or a completion since the last scan
        self._finished: list = []             # (slot, job) reported by workers
        self._stop = False
        self._error = None
        self.slots = [_Slot(self, torch, device, k) for k in range(slots)]
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
            r.seq = self._seq
            self._seq += 1
            self._inbox.append(r)
            self._dirty = True
            self._cv.notify()
        return r.future

    def close(self, wait: bool = True) -> None:
        with self._cv:
            self._stop = True
            self._dirty = True
            self._cv.notify()
        if wait:
            self._thread.join()
            for s in self.slots:
                s.thread.join()
        if self._error is not None:
            raise self._error

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- dispatch loop (all state below is touched by this thread only) ------
    def _completed(self, slot, job) -> None:
        """Called by a worker when its job is done."""
        with self._cv:
            self._finished.append((slot, job))
            self._dirty = True
            self._cv.notify()

    def _loop(self):
        try:
            while True:
                with self._cv:
                    while not self._dirty:
                        if self._stop and not self.queues and not any(s.busy for s in self.slots):
                            for s in self.slots:
                                s.jobs.put(None)
                            return
                        self._cv.wait()
                    self._dirty = False
                    finished, self._finished = self._finished, []
                    inbox, self._inbox = self._inbox, []
                for r in inbox:
                    q = self.queues.get(r.scene)
                    if q is None:
                        q = self.queues[r.scene] = collections.deque()
                    q.append(r)
                for slot, job in finished:
                    slot.busy = False
                    if job.err is None:
                        job.finish(job.out, job.t_done)
                    else:
                        job.fail(job.err, job.t_done)
                while self._dispatch():
                    pass
                if self.queues and not any(s.busy for s in self.slots):
                    self._unblock()
        except BaseException as exc:  # fail every waiting request, keep the cause
            self._error = exc
            with self._cv:
                rest = self._inbox
                self._inbox = []
            rest += [r for q in self.queues.values() for r in q]
            self.queues.clear()
            for r in rest:
                if not r.future.done():
                    r.future.set_exception(exc)
            for s in self.slots:
                s.jobs.put(None)

    def _unblock(self) -> None:
        """Nothing runs and nothing waiting was admitted: the oldest request
        can never be (it needs more memory than the budget frees)."""
        if not self.queues:
            return
        r = min((q[0] for q in self.queues.values()), key=lambda x: x.seq)
        self._reject(r, MemoryError(f"a {r.kind} of {r.data.shape[0]} rows does not fit the HBM budget "
                                    f"({self.budget} bytes)"))

    def _reject(self, r: Request, exc: BaseException) -> None:
        self._take([r])
        r.future.set_exception(exc)

    def _pending_scenes(self) -> set[int]:
        return set(self.queues)

    def _admissible(self, r: Request) -> bool:
        res = self.resident.get(r.scene)
        if r.scene in self.writing:
            return False
        if r.kind == TRACE:
            return res is not None
        if r.kind == REFIT:
            return res is not None and res.busy == 0
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
        """Starts one job on a free slot; False when nothing could start.
        Candidates are each scene's oldest waiting request (oldest scene
        first) and, for a trace, the run of traces queued right behind it,
        so a scene's requests start in submission order."""
        free = [s for s in self.slots if not s.busy]
        if not free or not self.queues:
            return False
        heads = sorted(self.queues.items(), key=lambda kv: kv[1][0].seq)
        chosen = None
        for scene, q in heads:
            r = q[0]
            res = self.resident.get(scene)
            if r.kind != BUILD and res is None and scene not in self.writing:
                self._reject(r, KeyError(f"scene {scene} is not resident"))
                return True
            if r.kind == REFIT and scene not in self.writing and res.n != r.data.shape[0]:
                self._reject(r, ValueError(f"refit of scene {scene} with {r.data.shape[0]} triangles; "
                                           f"it was built with {res.n}"))
                return True
            if self._admissible(r):
                chosen = r
                break
        if chosen is None:
            return False
        slot = free[0]
        if chosen.kind == BUILD:
            group = [chosen]
            if 2 <= chosen.data.shape[0] <= self.batch_max_tris:
                for scene, q in heads:
                    if len(group) >= self.batch_max_requests:
                        break
                    r = q[0]
                    if r is not chosen and r.kind == BUILD and 2 <= r.data.shape[0] <= self.batch_max_tris \
                            and self._admissible(r):
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
            group = self._trace_run(chosen.scene, [chosen])
            if res.batch is not None and len(group) < self.batch_max_requests \
                    and chosen.data.shape[0] <= self.trace_batch_max_rays:
                for scene, q in heads:
                    other = self.resident.get(scene)
                    if scene == chosen.scene or other is None or other.batch is not res.batch \
                            or scene in self.writing or q[0].kind != TRACE \
                            or q[0].data.shape[0] > self.trace_batch_max_rays:
                        continue
                    group = self._trace_run(scene, group + [q[0]])
                    if len(group) >= self.batch_max_requests:
                        break
            self._take(group)
            if len(group) > 1:
                self.coalesced += len(group)
            self._start_trace(slot, group)
        return True

    def _trace_run(self, scene: int, group: list) -> list:
        """Extends a group ending with the head of `scene`'s queue by the small
        traces queued right behind it (they read the same tree)."""
        if group[-1].data.shape[0] > self.trace_batch_max_rays:
            return group
        q = self.queues[scene]
        for k in range(1, len(q)):
            r = q[k]
            if len(group) >= self.batch_max_requests or r.kind != TRACE \
                    or r.data.shape[0] > self.trace_batch_max_rays:
                break
            group.append(r)
        return group

    def _take(self, group) -> None:
        """Removes a group from the queues: for each scene it is a run from
        the front of the scene's queue, in queue order."""
        now = time.perf_counter()
        for r in group:
            q = self.queues[r.scene]
            assert q[0] is r
            q.popleft()
            if not q:
                del self.queues[r.scene]
            r.started = now

    def _finish(self, group, t_done: float, results=None) -> None:
        for k, r in enumerate(group):
            r.done = t_done
            self.done.append(r)
            r.future.set_result(None if results is None else results[k])

    def _fail(self, group, exc: BaseException, t_done: float) -> None:
        for r in group:
            r.done = t_done
            if not r.future.done():
                r.future.set_exception(exc)

    def _launch(self, slot, work, finish, fail) -> None:
        slot.busy = True
        slot.jobs.put(_Job(work, finish, fail))

    # ---- jobs: bookkeeping here, GPU work in the slot's worker -----------------
    def _start_build(self, slot, r: Request) -> None:
        n = r.data.shape[0]
        nbytes = scene_bytes(n)
        self.used += nbytes
        self.writing.add(r.scene)
        L, ctx = _lib.lib(), slot.ctx

        def work():
            dev = slot.upload(r.data, 12)
            bvh = lbapi.BVH(ctx)
            ctx.check(L.lbvh_build_triangles(ctx.handle, dev.data_ptr(), n, 0, bvh.handle))
            # the traversal copy is made here, on this stream, so that traces
            # on other streams never build it concurrently
            ctx.check(L.lbvh_bvh_prepare_trace(ctx.handle, bvh.handle))
            bvh.kind = lbapi.TRIANGLES
            return bvh, dev

        def finish(out, t):
            bvh, dev = out
            self._drop(r.scene)
            self.resident[r.scene] = Resident(n, nbytes, bvh=bvh, tris=dev, last_use=t)
            self.writing.discard(r.scene)
            self._finish([r], t)

        def fail(exc, t):
            self.used -= nbytes
            self.writing.discard(r.scene)
            self._fail([r], exc, t)

        self._launch(slot, work, finish, fail)

    def _start_batch_build(self, slot, group) -> None:
        counts = np.array([r.data.shape[0] for r in group], np.int64)
        offsets = np.zeros(len(group) + 1, np.uint32)
        offsets[1:] = np.cumsum(counts)
        sizes = [scene_bytes(int(c)) for c in counts]
        for r, b in zip(group, sizes):
            self.used += b
            self.writing.add(r.scene)
        L, ctx, torch = _lib.lib(), slot.ctx, self.torch

        def work():
            dev = torch.empty((int(offsets[-1]), 12), dtype=torch.float32, device=self.device)
            for k, r in enumerate(group):
                dev[int(offsets[k]) : int(offsets[k + 1])].copy_(torch.from_numpy(r.data), non_blocking=True)
            batch = lbapi.Batch(ctx)
            ctx.check(L.lbvh_batch_build_triangles(ctx.handle, dev.data_ptr(), int(offsets[-1]),
                                                   offsets.ctypes.data, len(group), batch._h))
            ctx.check(L.lbvh_batch_prepare_trace(ctx.handle, batch._h))
            batch._keep = (dev, offsets)
            batch._offsets = offsets
            return batch, dev

        def finish(out, t):
            batch, dev = out
            ref = _BatchRef(batch, dev, offsets, members=len(group))
            for k, (r, b) in enumerate(zip(group, sizes)):
                self._drop(r.scene)
                self.resident[r.scene] = Resident(r.data.shape[0], b, batch=ref, index=k, last_use=t)
                self.writing.discard(r.scene)
            self._finish(group, t)

        def fail(exc, t):
            for r, b in zip(group, sizes):
                self.used -= b
                self.writing.discard(r.scene)
            self._fail(group, exc, t)

        self._launch(slot, work, finish, fail)

    def _start_refit(self, slot, r: Request) -> None:
        """A batch member is first moved into its own BVH (the same nodes,
        copied on the device), then refitted."""
        res = self.resident[r.scene]
        self.writing.add(r.scene)
        L, ctx, torch = _lib.lib(), slot.ctx, self.torch
        ref, k = res.batch, res.index

        def work():
            bvh = res.bvh
            if ref is not None:
                o = ref.offsets
                total_nodes = int(o[-1]) - (o.size - 1)
                all_nodes = torch.empty((total_nodes, 8), dtype=torch.float32, device=self.device)
                ctx.check(L.lbvh_batch_nodes(ctx.handle, ref.batch._h, all_nodes.data_ptr()))
                start = int(o[k]) - k
                nodes = all_nodes[start : start + int(o[k + 1] - o[k]) - 1]
                bvh = lbapi.BVH.from_nodes(nodes, ref.tris[int(o[k]) : int(o[k + 1])], ctx)
            dev = slot.upload(r.data, 12)
            ctx.check(L.lbvh_refit_triangles(ctx.handle, bvh.handle, dev.data_ptr()))
            ctx.check(L.lbvh_bvh_prepare_trace(ctx.handle, bvh.handle))
            return bvh, dev

        def finish(out, t):
            bvh, dev = out
            if ref is not None:  # the member leaves its batch
                ref.members -= 1
                if ref.members == 0:
                    ref.batch.close()
                cur = Resident(res.n, res.nbytes, bvh=bvh, tris=dev, last_use=t)
                self.resident[r.scene] = cur
            else:
                res.tris = dev  # the refitted BVH now borrows these triangles
                res.last_use = t
            self.resident.move_to_end(r.scene)
            self.writing.discard(r.scene)
            self._finish([r], t)

        def fail(exc, t):
            # the tree may be half refitted: the scene leaves residency
            self.writing.discard(r.scene)
            self._drop(r.scene)
            self._fail([r], exc, t)

        self._launch(slot, work, finish, fail)

    def _start_trace(self, slot, group) -> None:
        torch = self.torch
        used = [self.resident[r.scene] for r in group]
        for res in used:
            res.busy += 1
        res0 = used[0]
        L, ctx = _lib.lib(), slot.ctx
        if res0.batch is None:  # traces of one tree, one after another
            ends = np.cumsum([r.data.shape[0] for r in group])
            spans = [(int(e - r.data.shape[0]), int(e)) for r, e in zip(group, ends)]
            m = int(ends[-1])
            roff = None
        else:
            ref = res0.batch
            nm = ref.offsets.size - 1
            order = sorted(range(len(group)), key=lambda k: used[k].index)
            per_mesh = np.zeros(nm, np.int64)
            for k in order:
                per_mesh[used[k].index] += group[k].data.shape[0]
            roff = np.zeros(nm + 1, np.uint32)
            roff[1:] = np.cumsum(per_mesh)
            cursor = roff[:-1].astype(np.int64)
            spans = [None] * len(group)
            for k in order:
                idx = used[k].index
                spans[k] = (int(cursor[idx]), int(cursor[idx]) + group[k].data.shape[0])
                cursor[idx] += group[k].data.shape[0]
            m = int(roff[-1])

        def work():
            rays = torch.empty((m, 8), dtype=torch.float32, device=self.device)
            for (a, b), r in zip(spans, group):
                rays[a:b].copy_(torch.from_numpy(r.data), non_blocking=True)
            hits = torch.empty((m, 4), dtype=torch.float32, device=self.device)
            if m == 0:
                pass
            elif roff is None:
                ctx.check(L.lbvh_trace_triangles(ctx.handle, res0.bvh.handle, rays.data_ptr(), m, hits.data_ptr()))
            else:
                ctx.check(L.lbvh_batch_trace_triangles(ctx.handle, res0.batch.batch._h, rays.data_ptr(),
                                                       roff.ctypes.data, m, hits.data_ptr()))
            outs = []
            for a, b in spans:  # mapped while the trace runs
                out = np.empty(b - a, lbapi.HIT_DTYPE)
                _touch(out)
                outs.append(out)
            for (a, b), out in zip(spans, outs):
                torch.from_numpy(out.view(np.float32).reshape(-1, 4)).copy_(hits[a:b], non_blocking=True)
            return outs

        def settle(t):
            for r, res in zip(group, used):
                res.busy -= 1
                res.last_use = t
                if res.retired:
                    if res.busy == 0:
                        self._release(res)
                elif r.scene in self.resident:
                    self.resident.move_to_end(r.scene)

        def finish(outs, t):
            settle(t)
            self._finish(group, t, outs)

        def fail(exc, t):
            settle(t)
            self._fail(group, exc, t)

        self._launch(slot, work, finish, fail)


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
