"""Continuous-batching ray-query serving over HBM-resident scenes.

A request is a batch of rays (closest or any hit) against one scene; some requests bring a new
scene that must be built before their rays run.  Two servers process the same arrival trace:

* ``ContinuousServer`` — requests that have arrived wait in a queue; whenever one of ``slots``
  CUDA streams is free, ready work (scene resident) forms one batch of at most ``max_batch_rays``
  rays: requests with the fewest rays left go first (shortest remaining work; a request that has
  waited ``max_wait_s`` goes first regardless), and a request larger than what is left of the
  batch contributes a chunk of its rays and keeps the rest queued, so no launch holds the GPU
  for long and a small request never waits behind a whole large one.  The batch's rays are
  copied in, traced with one ``lcx_trace_jobs`` launch per query kind (each lane of the
  persistent kernel serves its ray's job), and copied back; a request completes with its last
  chunk.  Batches on different streams overlap on the device; the query streams have a higher
  priority than the build stream.  Scene builds run on their own thread and stream, so an
  upload never blocks admission.  Scenes live in an HBM budget with LRU eviction of scenes no
  queued or in-flight request needs; an evicted scene is rebuilt on demand.  Scenes resident before
  requests arrive are FAST_TRACE builds (binned SAH) and may use triangle splitting
  (``SceneStore.warm(split=...)``), which traces scenes of long overlapping triangles faster
  without putting its build cost on any request; builds on a request's path (uploads, rebuilds
  after an eviction) are FAST_BUILD builds (Morton LBVH, about half the build time).  On a coherent CPU-GPU link the kernels read each request's pinned rays and write its
  pinned results directly (``direct_host``), with no copies.
* ``PlainServer`` — one request at a time: build if needed, copy in, one trace call, copy out,
  wait, next.

Latency is arrival -> results in host memory.  No counterpart in the reference (its queries run
inside one user kernel per dispatch); the scenes, builds and queries are the Mesh/Accel path.
"""
from __future__ import annotations

import ctypes
import queue
import threading
import time
from collections import OrderedDict, deque
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from . import scenes as S
from .accel import HINT_FAST_BUILD, HINT_FAST_TRACE, Accel, AccelOption, Mesh, stream_handle


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the start of the run
    scene: int                # scene id
    rays: np.ndarray          # RAY_DTYPE
    any_hit: bool
    new_scene: S.MeshData | None = None  # uploaded (and built) before the rays run
    # filled in by the server
    dispatched: float = -1.0  # first launch of any of its rays (seconds after the start)
    done: float = -1.0
    result: np.ndarray | None = None
    error: str | None = None  # the request failed (its scene could not be admitted or built)
    cancelled: bool = False   # cancelled before all of its rays ran; its results are incomplete


@dataclass
class _Resident:
    mesh: object
    accel: Accel
    nbytes: int
    pins: int = 0


class BudgetError(RuntimeError):
    """A scene does not fit the HBM budget even with every unpinned scene evicted."""


class SceneStore:
    """Scenes by id: host data always, device BVHs within `budget_bytes` (LRU eviction).  A scene
    larger than the whole budget is refused (BudgetError) instead of overrunning it."""

    def __init__(self, scenes: dict, budget_bytes: int, request_hint: int = HINT_FAST_BUILD):
        self.host = dict(scenes)         # id -> MeshData
        self.budget = budget_bytes
        self.request_hint = request_hint  # AccelOption hint of builds on a request's path
        self.res: OrderedDict = OrderedDict()  # id -> _Resident, most recent last
        self.used = 0
        self.lock = threading.Lock()
        self.builds = 0
        self.evictions = 0

    def warm(self, ids, stream=None, split: float = 0.0) -> None:
        """Build scenes `ids` (as many as the budget holds) before serving starts.  split > 0: with
        triangle splitting at that fraction (lcx_set_build_split): slower builds, faster traces on
        scenes of long overlapping triangles; builds during serving (uploads, rebuilds after an
        eviction) keep the process's setting."""
        import torch
        stream = stream or torch.cuda.current_stream()
        lib = _capi.load()
        old = ctypes.c_float(0.0)
        _capi.check(lib.lcx_get_build_split(ctypes.byref(old)), "lcx_get_build_split")
        _capi.check(lib.lcx_set_build_split(ctypes.c_float(split)), "lcx_set_build_split")
        try:
            for sid in ids:
                self.build(sid, None, stream, hint=HINT_FAST_TRACE)
            torch.cuda.synchronize()
        finally:
            _capi.check(lib.lcx_set_build_split(old), "lcx_set_build_split")

    @staticmethod
    def estimate(md: S.MeshData) -> int:
        """Device bytes of a resident scene: uploaded buffers + BVH (~0.36 wide nodes x 288 B +
        48 B per triangle at leaf size 1)."""
        return md.vertices.nbytes + md.triangles.nbytes + md.tri_count * 160 + (1 << 16)

    def resident(self, sid: int) -> bool:
        with self.lock:
            return sid in self.res

    def pin(self, sid: int) -> _Resident:
        """Keep scene `sid` resident until unpin; returns its resident record."""
        with self.lock:
            r = self.res[sid]
            r.pins += 1
            self.res.move_to_end(sid)
            return r

    def try_pin(self, sid: int):
        """pin(sid) if the scene is resident, else None, in one step (no eviction in between)."""
        with self.lock:
            r = self.res.get(sid)
            if r is None:
                return None
            r.pins += 1
            self.res.move_to_end(sid)
            return r

    def unpin(self, r: _Resident):
        with self.lock:
            r.pins -= 1

    def _evict_for(self, need: int) -> list:
        """Under the lock: unregisters least recently used unpinned scenes until `need` bytes fit
        and returns them; the caller destroys them after releasing the lock (a destroy waits for
        the device, which must not hold up pin/try_pin)."""
        victims = []
        for sid in list(self.res.keys()):
            if self.used + need <= self.budget:
                break
            r = self.res[sid]
            if r.pins == 0:
                del self.res[sid]
                self.used -= r.nbytes
                self.evictions += 1
                victims.append(r)
        return victims

    @staticmethod
    def _destroy(victims: list):
        for r in victims:
            r.accel.destroy()
            r.mesh.destroy()

    def build(self, sid: int, data: S.MeshData | None, stream, hint: int | None = None) -> None:
        """Upload and build scene `sid` on `stream`; `data` registers a new scene under a new id
        (scene ids are never reused, so no request races a replacement).  hint: the AccelOption
        hint of the build (None: the store's request_hint)."""
        import torch
        if data is not None:
            with self.lock:
                if sid in self.host:
                    raise ValueError(f"scene id {sid} already exists")
                self.host[sid] = data
        md = self.host[sid]
        est = self.estimate(md)
        if est > self.budget:
            raise BudgetError(f"scene {sid} needs about {est} bytes of HBM; the budget is {self.budget}")
        with self.lock:
            victims = self._evict_for(est)
        self._destroy(victims)
        hv, ht = _pinned_mesh(md)
        with torch.cuda.stream(stream):  # asynchronous copies from pinned staging
            v = torch.empty(hv.shape, dtype=torch.float32, device="cuda")
            v.copy_(hv, non_blocking=True)
            t = torch.empty(ht.shape, dtype=torch.int32, device="cuda")
            t.copy_(ht, non_blocking=True)
        mesh = Mesh(v, t, AccelOption(hint=self.request_hint if hint is None else hint))
        mesh.build(stream=stream)
        acc = Accel()
        acc.emplace_back(mesh)
        acc.build(stream=stream)
        nbytes = est
        with self.lock:
            self.res[sid] = _Resident(mesh, acc, nbytes)
            self.used += nbytes
            self.builds += 1


class _Slot:
    def __init__(self, max_rays: int):
        import torch
        self.stream = torch.cuda.Stream(priority=-1)  # queries ahead of the build stream
        self.rays = torch.empty(max_rays * 8, dtype=torch.float32, device="cuda")
        self.hits = torch.empty(max_rays * 6, dtype=torch.int32, device="cuda")
        self.occ = torch.empty(max_rays, dtype=torch.uint8, device="cuda")
        self.event = None
        self.t_start = None  # timing event recorded before the batch's first copy
        self.batch = []


_PIN_CACHE: dict = {}


def _pinned(a: np.ndarray):
    """Pinned host copy of a ray array (shared by the requests that reuse it)."""
    import torch
    key = id(a)
    hit = _PIN_CACHE.get(key)
    if hit is not None and hit[0] is a:
        return hit[1]
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).pin_memory()
    _PIN_CACHE[key] = (a, t)
    return t


_PIN_MESH: dict = {}


def _pinned_mesh(md: S.MeshData):
    """Pinned host copies of a scene's vertices (float32) and indices (as int32, same bits):
    where a server receives uploads, so the device copies are asynchronous."""
    import torch
    hit = _PIN_MESH.get(id(md))
    if hit is not None and hit[0] is md:
        return hit[1], hit[2]
    v = torch.from_numpy(np.ascontiguousarray(md.vertices, np.float32)).pin_memory()
    t = torch.from_numpy(np.ascontiguousarray(md.triangles).view(np.int32)).pin_memory()
    _PIN_MESH[id(md)] = (md, v, t)
    return v, t


class ContinuousServer:
    # Defaults measured on GB300 (64 displaced-mesh scenes, 800 requests/s): 1M-ray launches with
    # at most 2M rays in flight gave the lowest p99 for 0.5M-2M-ray queries (11-13 ms, against
    # 22 ms for 2M-ray launches without an in-flight bound); serialising the kernels was worse.
    def __init__(self, store: SceneStore, slots: int = 4, max_batch_rays: int = 1 << 20, layout: int = 1,
                 max_wait_s: float = 0.05, min_chunk: int = 1 << 16, max_inflight_rays: int | None = 2 << 20,
                 build_priority: int = 0, max_concurrent_kernels: int | None = None,
                 max_batch_ms: float | None = None, direct_host: bool | None = None, on_launch=None):
        self.store = store
        # on_launch(server, batch): called by the serving loop after each launch, with the batch's
        # (request, first ray, rays) pieces (progress reporting, or cancelling from the loop itself)
        self.on_launch = on_launch
        self._cancel = set()
        self._cancel_lock = threading.Lock()
        self.failed = 0
        self.cancelled = 0
        # direct host access: on a coherent CPU-GPU link (NVLink-C2C) the trace kernel reads each
        # request's pinned rays and writes its pinned results itself, with no copies in or out;
        # None = when the device has such a link (lcx_get_host_access)
        if direct_host is None:
            mode, coherent = ctypes.c_uint32(0), ctypes.c_uint32(0)
            _capi.check(_capi.load().lcx_get_host_access(ctypes.byref(mode), ctypes.byref(coherent)),
                        "lcx_get_host_access")
            direct_host = bool(coherent.value)
        self.direct_host = direct_host
        # cost-aware chunking: a request contributes at most max_batch_ms of estimated GPU time to a
        # batch, by its scene's measured cost per ray (an EWMA over completed batches); None = off.
        # Measured on the 800 req/s mix: p99 of 0.5M-2M-ray queries 10.1-11.3 ms off, 22-39 ms at
        # 0.6-2.5 ms caps (more, smaller launches cost more per-batch overhead than they save in
        # waiting behind long batches), so it stays off.
        self.max_batch_ms = max_batch_ms
        self.ns_per_ray: dict = {}
        self.lib = _capi.load()
        self.layout = layout
        self.max_batch_rays = max_batch_rays
        # rays launched and not yet complete, over all slots: bounds how much work a new
        # request can find ahead of it on the device
        self.max_inflight_rays = max_inflight_rays or slots * max_batch_rays
        self.build_priority = build_priority
        # trace kernels allowed to run at once: a batch's kernel waits for the kernel launched
        # this many batches before it (copies of every slot still overlap); None = no limit
        self.max_concurrent_kernels = max_concurrent_kernels
        self._kernel_events = deque()
        self.inflight = 0
        self.max_wait_s = max_wait_s
        self.min_chunk = min_chunk
        self.slots = [_Slot(max_batch_rays) for _ in range(slots)]
        self.build_q: queue.Queue = queue.Queue()
        self.built: queue.Queue = queue.Queue()
        self.batches = 0
        self.chunks = 0
        self.trace_launches = 0  # lcx_trace_jobs launches one kernel per query kind in a batch
        # per batch: (launch time, completion time seen by the loop, [(request id, first ray, rays)])
        self.timeline = []

    def cancel(self, rid: int) -> None:
        """Cancel request `rid` (from any thread, before or while it runs).  Rays not yet launched
        are dropped; launched chunks finish (a kernel is not interrupted), then the request
        completes with ``cancelled`` set and incomplete results.  Other requests are unaffected."""
        with self._cancel_lock:
            self._cancel.add(rid)

    def _builder(self):
        import torch
        stream = torch.cuda.Stream(priority=self.build_priority)  # 0: below the query streams (-1)
        while True:
            item = self.build_q.get()
            if item is None:
                return
            sid, data = item
            try:
                self.store.build(sid, data, stream)
                torch.cuda.current_stream().wait_stream(stream)
                stream.synchronize()
                self.built.put((sid, None))
            except Exception as e:  # reported to the loop
                self.built.put((sid, e))

    def _take(self, pending: list, now: float):
        """The next batch: (request, first ray, ray count) pieces, fewest remaining rays first
        (requests waiting longer than max_wait_s before all others), at most max_batch_rays and
        at most what max_inflight_rays leaves."""
        cap = min(self.max_batch_rays, self.max_inflight_rays - self.inflight)
        if cap < min(self.min_chunk, self.max_batch_rays):
            return []
        ready = sorted(pending, key=lambda r: (now - r.arrival < self.max_wait_s, r.rays.shape[0] - r._next,
                                               r.arrival))
        batch, total = [], 0
        for r in ready:
            room = cap - total
            left = r.rays.shape[0] - r._next
            if room <= 0:
                break
            if left > room and room < self.min_chunk and batch:
                continue
            pin = self.store.try_pin(r.scene)  # pinned with the selection: cannot be evicted in between
            if pin is None:
                continue
            r._pins.append(pin)
            n = min(left, room)
            if self.max_batch_ms is not None:  # at most max_batch_ms of this scene's estimated work
                est = self.ns_per_ray.get(r.scene, 1.0)
                n = min(n, max(self.min_chunk, int(self.max_batch_ms * 1e6 / est)))
            batch.append((r, r._next, n))
            r._next += n
            r._out += 1
            total += n
        return batch

    def run(self, requests: list) -> list:
        import torch
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            r._h_rays = _pinned(r.rays)
            r._h_out = torch.empty(r.rays.shape[0] * (1 if r.any_hit else 24), dtype=torch.uint8).pin_memory()
            r._next, r._out, r._pins = 0, 0, []
            if r.new_scene is not None:
                _pinned_mesh(r.new_scene)
        builder = threading.Thread(target=self._builder, daemon=True)
        builder.start()
        pending = []            # arrived, with rays not yet dispatched
        building = set()        # scene ids being built
        waiting_new = {}        # scene id -> requests whose new scene is being uploaded
        nxt = 0
        done = 0
        t0 = time.perf_counter()
        try:
            while done < len(reqs):
                progressed = False
                now = time.perf_counter() - t0
                # cancellations: drop the unlaunched rays of cancelled requests
                with self._cancel_lock:
                    cancel = set(self._cancel)
                if cancel:
                    keep = []
                    for r in pending:
                        if r.rid in cancel and not r.cancelled:
                            r.cancelled = True
                            self.cancelled += 1
                            r._next = r.rays.shape[0]
                            if r._out == 0:  # nothing in flight: done now
                                r.done = now
                                done += 1
                            progressed = True
                        else:
                            keep.append(r)
                    pending = keep
                # arrivals
                while nxt < len(reqs) and reqs[nxt].arrival <= now:
                    r = reqs[nxt]
                    nxt += 1
                    if r.rid in cancel:  # cancelled before it arrived
                        r.cancelled = True
                        self.cancelled += 1
                        r.done = now
                        done += 1
                        continue
                    if r.new_scene is not None:
                        waiting_new.setdefault(r.scene, []).append(r)
                        if r.scene not in building:
                            building.add(r.scene)
                            self.build_q.put((r.scene, r.new_scene))
                    else:
                        pending.append(r)
                # finished builds
                while True:
                    try:
                        sid, err = self.built.get_nowait()
                    except queue.Empty:
                        break
                    progressed = True
                    building.discard(sid)
                    if err is not None:
                        if not isinstance(err, BudgetError):
                            raise err
                        # the scene cannot be admitted: its requests fail, the others go on
                        failed = waiting_new.pop(sid, []) + [r for r in pending if r.scene == sid]
                        pending = [r for r in pending if r.scene != sid]
                        for r in failed:
                            r.error = str(err)
                            r.done = time.perf_counter() - t0
                            self.failed += 1
                            done += 1
                        continue
                    pending.extend(waiting_new.pop(sid, []))
                # completed batches
                for sl in self.slots:
                    if sl.event is not None and sl.event.query():
                        t = time.perf_counter() - t0
                        if self.max_batch_ms is not None and sl.t_start is not None:
                            ms = sl.t_start.elapsed_time(sl.event)
                            rays = sum(n for _, _, n in sl.batch)
                            if rays > 0 and ms > 0.0:
                                v = ms * 1e6 / rays
                                for sc in {r.scene for r, _, _ in sl.batch}:
                                    old = self.ns_per_ray.get(sc)
                                    self.ns_per_ray[sc] = v if old is None else 0.7 * old + 0.3 * v
                        for r, _, n in sl.batch:
                            self.store.unpin(r._pins.pop())
                            self.inflight -= n
                            r._out -= 1
                            if r._out == 0 and r._next == r.rays.shape[0]:
                                r.done = t
                                done += 1
                        self.timeline.append((sl.t_launch, t, [(r.rid, f, n) for r, f, n in sl.batch]))
                        progressed = True
                        sl.event = None
                        sl.batch = []
                # scenes evicted while queued: rebuild on demand
                for r in pending:
                    if not self.store.resident(r.scene) and r.scene not in building:
                        building.add(r.scene)
                        self.build_q.put((r.scene, None))
                # dispatch: one batch per free slot
                for sl in self.slots:
                    if sl.event is not None or not pending:
                        continue
                    batch = self._take(pending, time.perf_counter() - t0)
                    if not batch:
                        break
                    pending = [r for r in pending if r._next < r.rays.shape[0]]
                    self._launch(sl, batch, time.perf_counter() - t0)
                    self.batches += 1
                    self.chunks += len(batch)
                    progressed = True
                    if self.on_launch is not None:
                        self.on_launch(self, batch)
                if not progressed:
                    time.sleep(20e-6)  # let the builder thread run (GIL) while waiting
        finally:
            self.build_q.put(None)
            builder.join(timeout=30)
        return reqs

    def _launch(self, sl: _Slot, batch: list, now: float = -1.0):
        import torch
        jobs = (_capi.LcxTraceJob * len(batch))()
        for r, _, n in batch:
            self.inflight += n
            if r.dispatched < 0:
                r.dispatched = now
        with torch.cuda.stream(sl.stream):
            if self.max_batch_ms is not None:
                sl.t_start = torch.cuda.Event(enable_timing=True)
                sl.t_start.record(sl.stream)
            off = 0
            outs = []
            for i, (r, first, n) in enumerate(batch):
                pin = r._pins[-1]
                k = 1 if r.any_hit else 24
                if self.direct_host:  # the kernel reads and writes the request's pinned buffers
                    jobs[i] = _capi.LcxTraceJob(pin.accel.handle, r._h_rays.data_ptr() + first * 32,
                                                r._h_out.data_ptr() + first * k, n, 0xFF, 1 if r.any_hit else 0, 0)
                    continue
                seg = sl.rays[off * 8:(off + n) * 8]
                seg.view(torch.uint8).copy_(r._h_rays[first * 32:(first + n) * 32], non_blocking=True)
                out = sl.occ[off:off + n] if r.any_hit else sl.hits[off * 6:(off + n) * 6]
                jobs[i] = _capi.LcxTraceJob(pin.accel.handle, seg.data_ptr(), out.data_ptr(), n, 0xFF,
                                            1 if r.any_hit else 0, 0)
                outs.append((r._h_out[first * k:(first + n) * k], out))
                off += n
            k = self.max_concurrent_kernels
            if k is not None and len(self._kernel_events) >= k:
                sl.stream.wait_event(self._kernel_events[-k])
            _capi.check(self.lib.lcx_trace_jobs(jobs, len(batch), self.layout, stream_handle(sl.stream)),
                        "lcx_trace_jobs")
            if k is not None:
                ev = torch.cuda.Event()
                ev.record(sl.stream)
                self._kernel_events.append(ev)
                while len(self._kernel_events) > k:
                    self._kernel_events.popleft()
            self.trace_launches += len({r.any_hit for r, _, _ in batch})
            for host, dev in outs:
                host.copy_(dev.view(torch.uint8), non_blocking=True)
            sl.event = torch.cuda.Event(enable_timing=self.max_batch_ms is not None)
            sl.event.record(sl.stream)
        sl.batch = batch
        sl.t_launch = now


class PlainServer:
    """One request at a time on one stream (the baseline)."""

    def __init__(self, store: SceneStore, layout: int = 1):
        self.store = store
        self.layout = layout

    def run(self, requests: list) -> list:
        import torch
        from .accel import rays_to_device
        reqs = sorted(requests, key=lambda r: r.arrival)
        stream = torch.cuda.Stream()
        for r in reqs:
            r._h_rays = _pinned(r.rays)
            r._h_out = torch.empty(r.rays.shape[0] * (1 if r.any_hit else 24), dtype=torch.uint8).pin_memory()
            if r.new_scene is not None:
                _pinned_mesh(r.new_scene)
        t0 = time.perf_counter()
        for r in reqs:
            while time.perf_counter() - t0 < r.arrival:
                pass
            if r.new_scene is not None or not self.store.resident(r.scene):
                try:
                    self.store.build(r.scene, r.new_scene, stream)
                except BudgetError as e:  # the request fails; the next one goes on
                    r.error = str(e)
                    r.done = time.perf_counter() - t0
                    continue
            pin = self.store.pin(r.scene)
            acc = pin.accel
            with torch.cuda.stream(stream):
                d = torch.empty(r.rays.shape[0] * 8, dtype=torch.float32, device="cuda")
                d.view(torch.uint8).copy_(r._h_rays, non_blocking=True)
                d = d.view(-1, 8)
                if r.any_hit:
                    out = acc.trace_any(d, layout=self.layout, stream=stream)
                else:
                    out = acc.trace_closest(d, layout=self.layout, stream=stream)
                r._h_out.copy_(out.view(torch.uint8).reshape(-1), non_blocking=True)
            stream.synchronize()
            self.store.unpin(pin)
            r.done = time.perf_counter() - t0
        return reqs


def results(reqs: list) -> list:
    """Per-request results as numpy (TriangleHit records or occlusion bytes)."""
    out = []
    for r in reqs:
        a = r._h_out.numpy()
        out.append(a.copy() if r.any_hit else a.view(S.HIT_DTYPE).copy())
    return out


def latency_stats(reqs: list) -> dict:
    """p50/p99 latency (ms) overall, for queries on resident scenes, for requests that upload a
    scene, and for 0.5M..2M-ray queries; aggregate Grays/s over the run.  Failed and cancelled
    requests are left out."""
    reqs = [r for r in reqs if r.error is None and not r.cancelled]
    lat = np.array([r.done - r.arrival for r in reqs]) * 1e3
    rays = np.array([r.rays.shape[0] for r in reqs])
    up = np.array([r.new_scene is not None for r in reqs])
    mid = (rays >= 500_000) & (rays <= 2_000_000) & ~up
    span = max(r.done for r in reqs) - min(r.arrival for r in reqs)

    def pct(mask, q):
        return float(np.percentile(lat[mask], q)) if mask.any() else None

    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()),
            "queries": {"p50_ms": pct(~up, 50), "p99_ms": pct(~up, 99), "count": int((~up).sum())},
            "uploads": {"p50_ms": pct(up, 50), "p99_ms": pct(up, 99), "count": int(up.sum())},
            "queries_0.5M_to_2M_rays": {"p50_ms": pct(mid, 50), "p99_ms": pct(mid, 99), "count": int(mid.sum())},
            "requests": len(reqs), "rays": int(rays.sum()), "span_s": span,
            "grays_per_s": float(rays.sum() / span / 1e9)}


def make_workload(n_scenes=64, n_requests=2000, rate_hz=1000.0, tri_lo=10_000, tri_hi=4_000_000,
                  ray_lo=1_000, ray_hi=4_000_000, new_scene_frac=0.08, seed=11, ray_pool=0):
    """Scenes log-uniform in [tri_lo, tri_hi] triangles (generated like the batched-build meshes);
    Poisson arrivals at rate_hz; ray counts log-uniform in [ray_lo, ray_hi], half camera rays and
    half sphere-uniform rays, half closest and half any; new_scene_frac of requests upload a new
    scene (under a fresh id).  ray_pool > 0 draws each request's rays from that many pre-generated
    sets per kind (bounded host memory for long runs)."""
    rng = np.random.default_rng(seed)
    tri = np.exp(rng.uniform(np.log(tri_lo), np.log(tri_hi), n_scenes)).astype(np.int64)
    scenes = {i: S.displaced_mesh(int(t), rng) for i, t in enumerate(tri)}
    arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, n_requests))
    counts = np.exp(rng.uniform(np.log(ray_lo), np.log(ray_hi), n_requests)).astype(np.int64)

    def make_rays(n, coherent, seed_):
        if coherent:
            w = max(1, int(np.sqrt(n)))
            return S.camera_rays(w, (n + w - 1) // w, eye=(0.0, 0.0, 3.5), seed=seed_)[:n]
        return S.sphere_rays(n, [-1.3, -1.3, -1.3], [1.3, 1.3, 1.3], seed=seed_)

    pool = None
    if ray_pool > 0:
        sizes = np.exp(np.linspace(np.log(ray_lo), np.log(ray_hi), ray_pool)).astype(np.int64)
        pool = {c: [make_rays(int(n), c, 1000 + 2 * i + int(c)) for i, n in enumerate(sizes)] for c in (0, 1)}
    reqs = []
    for k in range(n_requests):
        sid = int(rng.integers(0, n_scenes))
        n = int(counts[k])
        coherent = rng.random() < 0.5
        if pool is None:
            rays = make_rays(n, coherent, int(rng.integers(1 << 30)))
        else:
            sets = pool[int(coherent)]
            rays = sets[int(np.argmin([abs(np.log(s.shape[0] / n)) for s in sets]))]
        new = None
        if rng.random() < new_scene_frac:  # a new scene under a fresh id, built before the rays run
            new = S.displaced_mesh(int(tri[sid]), rng)
            sid = n_scenes + k
        reqs.append(Request(k, float(arrivals[k]), sid, rays, bool(rng.random() < 0.5), new))
    return scenes, reqs
