"""Continuous-batching render server over resident scenes.

Scenes stay resident on the device (the Store's role). Requests (scene,
camera, size) queue in arrival order; each of ``lanes`` pipelines owns a CUDA
stream, and whenever a lane is free the server admits queued requests into its
next batch while the batch's workspace estimate fits the lane's share of the
memory budget. Batches on different lanes overlap on the device; requests that
arrive while others are rendering join the next free lane's batch.

A request's workspace estimate is its padded ordinal count times the
per-ordinal workspace plus its expected intersections times the per-record
workspace; intersections are learned per (scene, size) from completed batches
(the largest per-view demand seen, with the reference's 1.25 headroom), seeded
by one probe render. A batch that overflows its intersection capacity is grown
with the reference's capacity policy (IntersectionCapacityPolicy.ts:90-100)
and rendered again, so no truncated image is ever returned.

Every request's image is the same as a render of that request alone: views of
a batch are independent (see gs3d_pipeline_render_batch).
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

from . import TiledGaussianPipeline, make_camera

# Workspace bytes per padded ordinal (projected mean/conic/colour 48, packed
# raster record 32, counts, keys, offsets 20, depth records x2 16) and per
# intersection record (tile ids and ordinals, ping-pong: 16).
BYTES_PER_ITEM = 116
BYTES_PER_RECORD = 16


@dataclass
class Request:
    rid: int
    scene: str
    frame: dict
    arrival: float = 0.0
    dispatched: float = 0.0
    completed: float = 0.0
    color: object = None
    attempts: int = 0

    @property
    def latency_ms(self) -> float:
        return 1000.0 * (self.completed - self.arrival)


@dataclass
class _Lane:
    pipe: TiledGaussianPipeline
    stream: object
    capacity: int
    batch: list = field(default_factory=list)
    event: object = None


class RenderServer:
    def __init__(self, scenes: dict, lanes: int = 2, budget_bytes: float = 40e9, max_views: int = 16,
                 precision: str = "half2", initial_capacity: int = 1 << 22):
        import torch
        self.scenes = scenes  # name -> device.DeviceScene
        self.budget = float(budget_bytes)
        self.max_views = int(max_views)
        self.queue = collections.deque()
        self.completed = []
        self.demand = {}  # (scene, w, h) -> intersections per view
        first = next(iter(scenes.values()))
        self.lanes = []
        for _ in range(lanes):
            pipe = TiledGaussianPipeline(first.data(), {"raster_precision": precision,
                                                        "intersection_capacity": initial_capacity})
            self.lanes.append(_Lane(pipe, torch.cuda.Stream(), initial_capacity))
        self.lane_budget = self.budget / lanes
        self.batches = 0
        self.retries = 0

    # -- estimates ----------------------------------------------------------
    def _key(self, req: Request):
        return (req.scene, int(req.frame["width"]), int(req.frame["height"]))

    def request_bytes(self, req: Request) -> int:
        sc = self.scenes[req.scene]
        items = (sc.active_count + 255) // 256 * 256
        inter = self.demand.get(self._key(req), 0)
        return items * BYTES_PER_ITEM + int(inter * 1.25) * BYTES_PER_RECORD

    def probe(self, frames_by_key: dict) -> None:
        """One render per (scene, size) to seed the demand estimates."""
        for (scene, w, h), frame in frames_by_key.items():
            req = Request(-1, scene, frame)
            self._render_batch(self.lanes[0], [req], record=False)
            self.lanes[0].event.synchronize()
            self._finish(self.lanes[0], time.perf_counter(), record=False)

    # -- dispatch -----------------------------------------------------------
    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _render_batch(self, lane: _Lane, batch: list, record: bool = True) -> None:
        import torch
        views = []
        need = 0
        for r in batch:
            sc = self.scenes[r.scene]
            W, H = int(r.frame["width"]), int(r.frame["height"])
            if r.color is None:
                r.color = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
            views.append((sc.data(), make_camera(r.frame), W, H, r.color.data_ptr(), 0, "rgba16f"))
            need += int(self.demand.get(self._key(r), 0) * 1.25)
            r.attempts += 1
        if need > lane.capacity:
            lane.capacity = (need + 255) // 256 * 256
            lane.pipe.resize_intersections(lane.capacity)
        with torch.cuda.stream(lane.stream):
            lane.pipe.render_batch(views, stream=lane.stream.cuda_stream)
            lane.event = torch.cuda.Event()
            lane.event.record(lane.stream)
        lane.batch = batch
        if record:
            self.batches += 1

    def _finish(self, lane: _Lane, now: float, record: bool = True) -> None:
        stats = lane.pipe.read_stats()
        batch = lane.batch
        lane.batch, lane.event = [], None
        if stats["overflow"]:
            # Never publish a truncated set: grow and render the batch again.
            lib = lane.pipe._lib
            grown = int(lib.gs3d_capacity_next(1 << 31, 2.0, 1.25, lane.capacity, stats["requestedIntersections"]))
            lane.capacity = max(grown, stats["requestedIntersections"] + 256)
            lane.pipe.resize_intersections(lane.capacity)
            self.retries += 1
            per_view = stats["requestedIntersections"] / max(1, len(batch))
            for r in batch:
                self.demand[self._key(r)] = max(self.demand.get(self._key(r), 0), per_view)
            self._render_batch(lane, batch, record)
            return
        per_view = stats["intersectionCount"] / max(1, len(batch))
        for r in batch:
            k = self._key(r)
            self.demand[k] = max(self.demand.get(k, 0), per_view)
            r.completed = now
            if record:
                self.completed.append(r)

    def poll(self, now: float) -> int:
        """Retire finished batches and start new ones; returns lanes busy."""
        busy = 0
        for lane in self.lanes:
            if lane.event is not None and lane.event.query():
                self._finish(lane, now)
            if lane.event is None and self.queue:
                batch, total = [], 0
                while self.queue and len(batch) < self.max_views:
                    nxt = self.queue[0]
                    b = self.request_bytes(nxt)
                    if batch and total + b > self.lane_budget:
                        break
                    self.queue.popleft()
                    nxt.dispatched = now
                    batch.append(nxt)
                    total += b
                # Requests of one scene side by side: consecutive views of a
                # scene share the projection's decode (a view group); every
                # request's image is unchanged by its place in the batch.
                batch.sort(key=lambda r: r.scene)
                self._render_batch(lane, batch)
            busy += lane.event is not None
        return busy

    def _wait_oldest(self) -> None:
        """Block until the batch dispatched first among the busy lanes is done
        (instead of spinning on event queries while nothing can be
        dispatched)."""
        busy = [l for l in self.lanes if l.event is not None]
        if busy:
            min(busy, key=lambda l: min(r.dispatched for r in l.batch) if l.batch else 0.0).event.synchronize()

    def run_closed(self, make_request, concurrency: int, total: int, warmup: int = 0) -> dict:
        """Closed loop: keep `concurrency` requests outstanding (each completed
        request is replaced at once by a new one from make_request(i)) until
        `total` have completed after `warmup` unrecorded ones. By Little's law
        the mean latency is concurrency / throughput."""
        self.completed = []
        self.batches = self.retries = 0
        issued = 0
        done = 0

        def submit_one():
            nonlocal issued
            r = make_request(issued)
            r.arrival = time.perf_counter()
            self.submit(r)
            issued += 1

        for _ in range(concurrency):
            submit_one()
        t0 = None
        recorded = []
        while done < warmup + total:
            now = time.perf_counter()
            before = len(self.completed)
            self.poll(now)
            finished = self.completed[before:]
            for r in finished:
                done += 1
                if done == warmup:
                    t0 = time.perf_counter()
                if done > warmup:
                    recorded.append(r)
                if issued < warmup + total:
                    submit_one()
            if not finished:
                # poll() has dispatched whatever a free lane could take, so
                # nothing can start before a batch completes: wait for one.
                self._wait_oldest()
        t1 = time.perf_counter()
        t0 = t0 if t0 is not None else t1
        lat = sorted(r.latency_ms for r in recorded)
        while any(l.event is not None for l in self.lanes):
            self.poll(time.perf_counter())
        fps = len(recorded) / (t1 - t0) if t1 > t0 else 0.0
        return {
            "concurrency": concurrency, "requests": len(recorded), "seconds": t1 - t0, "frames_per_s": fps,
            "p50_ms": lat[len(lat) // 2] if lat else None,
            "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))] if lat else None,
            "max_ms": lat[-1] if lat else None, "mean_ms": sum(lat) / len(lat) if lat else None,
            "little_bound_ms": 1000.0 * concurrency / fps if fps else None,
            "batches": self.batches, "retries": self.retries,
        }

    def run(self, requests: list, realtime: bool = True) -> dict:
        """Feed requests at their arrival times (seconds from start) and run
        until all complete. Returns latency and throughput statistics."""
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        for r in pending:
            r.arrival += t0
        i = 0
        while i < len(pending) or self.queue or any(l.event is not None for l in self.lanes):
            now = time.perf_counter()
            while i < len(pending) and (pending[i].arrival <= now or not realtime):
                if not realtime:
                    pending[i].arrival = now
                self.submit(pending[i])
                i += 1
            self.poll(now)
        t1 = time.perf_counter()
        lat = sorted(r.latency_ms for r in self.completed)
        return {
            "requests": len(self.completed), "seconds": t1 - t0,
            "frames_per_s": len(self.completed) / (t1 - t0) if t1 > t0 else 0.0,
            "p50_ms": lat[len(lat) // 2] if lat else None,
            "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))] if lat else None,
            "max_ms": lat[-1] if lat else None, "batches": self.batches, "retries": self.retries,
        }

    def close(self) -> None:
        for lane in self.lanes:
            lane.pipe.dispose()
