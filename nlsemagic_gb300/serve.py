"""Continuous-batching request loop over the batched persistent launch.

Requests (solves with their own dimension, grid, step count and precision
class) arrive over time.  The loop:

1. admits arrived requests, first come first served, while the device pool
   (the HBM budget) has room; state and potential are uploaded once and stay
   resident until the request completes;
2. advances every admitted solve by up to ``chunk_steps`` RK4 steps in one
   persistent launch (:meth:`nlsemagic_gb300.api.Batch.run`), so requests
   that arrived at different times share the device;
3. retires finished requests: the final state is downloaded as the snapshot
   returned to the caller and the slot's memory is released.

Latency of a request = completion time - arrival time.  The loop reports
p50 / p99 latency, queueing delay and the aggregate grid-point-steps/s.
There is no reference counterpart (NLSEmagic integrates one solve per call).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .api import Batch
from ._lib import NLSE_ERR_CAPACITY, NLSEError


@dataclass
class Completed:
    rid: int
    arrival: float
    admitted: float
    done: float
    points: int
    steps: int
    precision: int
    snapshot: np.ndarray = field(repr=False, default=None)

    @property
    def latency(self):
        return self.done - self.arrival


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs, dtype=float), q)) if len(xs) else float("nan")


class Server:
    def __init__(self, pool_bytes, chunk_steps=64, max_solves=8192, keep_snapshots=False):
        self.batch = Batch(pool_bytes, max_solves)
        self.pool_bytes = int(pool_bytes)
        self.chunk_steps = int(chunk_steps)
        self.keep_snapshots = keep_snapshots

    def close(self):
        self.batch.close()

    def serve(self, requests, time_scale=1.0, max_wall=None):
        """Serve `requests` (objects with .rid, .arrival seconds, .inst with
        U, V, s, a, h, BC, method, k, steps, precision) in real time.
        Arrival times are multiplied by time_scale.  Returns a summary dict
        and the list of Completed records."""
        b = self.batch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting = deque()
        active = {}
        done = []
        rejected = []
        t0 = time.perf_counter()
        busy = 0.0
        launches = 0
        while pending or waiting or active:
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                break
            while pending and pending[0].arrival * time_scale <= now:
                waiting.append(pending.popleft())
            # admission by the pool budget, in arrival order
            while waiting:
                r = waiting[0]
                i = r.inst
                need = Batch.bytes_for(i.U.shape, i.precision)
                if need > self.pool_bytes:
                    rejected.append(r.rid)
                    waiting.popleft()
                    continue
                try:
                    slot = b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, i.method,
                                 i.precision)
                except NLSEError as e:
                    if e.code == NLSE_ERR_CAPACITY:
                        break  # wait for memory to free up
                    raise
                active[slot] = (r, time.perf_counter() - t0)
                waiting.popleft()
            if not active:
                if pending:
                    dt = pending[0].arrival * time_scale - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                continue
            ts = time.perf_counter()
            b.run(self.chunk_steps)
            b.sync()
            busy += time.perf_counter() - ts
            launches += b.last_launches
            tnow = time.perf_counter() - t0
            for slot in list(active):
                if b.remaining(slot) == 0:
                    r, tadm = active.pop(slot)
                    snap = b.download(slot)
                    tdone = time.perf_counter() - t0
                    done.append(Completed(r.rid, r.arrival * time_scale, tadm, tdone,
                                          int(r.inst.U.size), int(r.inst.steps),
                                          int(r.inst.precision),
                                          snap if self.keep_snapshots else None))
                    b.remove(slot)
            del tnow
        wall = time.perf_counter() - t0
        lat = [c.latency for c in done]
        qd = [c.admitted - c.arrival for c in done]
        pts = float(sum(c.points * c.steps for c in done))
        summary = {
            "requests": len(done), "rejected": len(rejected), "wall_s": wall, "busy_s": busy,
            "launches": launches, "p50_latency_s": percentile(lat, 50),
            "p99_latency_s": percentile(lat, 99), "p50_queue_s": percentile(qd, 50),
            "p99_queue_s": percentile(qd, 99), "gpt_steps_per_s": pts / wall / 1e9 if wall else 0,
            "gpt_steps_per_busy_s": pts / busy / 1e9 if busy else 0, "point_steps": pts,
        }
        return summary, done


def serve_sequential(requests):
    """Baseline: one solve at a time, each through a resident Solver with
    graph-captured chunks (the reference's one-call-per-solve model, without
    its per-call allocation)."""
    from .api import Solver
    t0 = time.perf_counter()
    lat = []
    pts = 0.0
    clock = 0.0
    for r in sorted(requests, key=lambda r: r.arrival):
        i = r.inst
        start = max(clock, r.arrival)
        ts = time.perf_counter()
        s = Solver(i.U.shape, method=i.method, precision=i.precision, BC=i.BC, s=i.s, a=i.a,
                   h2=i.h * i.h, k=i.k)
        s.upload(i.U, i.V)
        s.run(i.steps)
        s.download()
        s.close()
        dt = time.perf_counter() - ts
        clock = start + dt
        lat.append(clock - r.arrival)
        pts += float(i.U.size) * i.steps
    wall = time.perf_counter() - t0
    return {"requests": len(lat), "busy_s": wall, "p50_latency_s": percentile(lat, 50),
            "p99_latency_s": percentile(lat, 99), "gpt_steps_per_busy_s": pts / wall / 1e9}
