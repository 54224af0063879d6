"""Continuous-batching request loop.

Requests (solves with their own dimension, grid, step count and precision
class) arrive over time.  The loop:

1. admits arrived requests, first come first served, while device memory
   allows.  Small solves (1D, 2D, and 3D below ``solo_points``) take a slot
   in the batched persistent launch (:class:`~nlsemagic_gb300.api.Batch`,
   admitted by its pool budget); large 3D solves get a resident
   :class:`~nlsemagic_gb300.api.Solver` of their own, which uses the tiled 3D
   stage kernels (admitted against ``solo_bytes``).  State and potential are
   uploaded once and stay resident until the request completes;
2. advances every admitted solve by up to ``chunk_steps`` RK4 steps per round:
   one persistent launch per precision class for all batched solves, and one
   graph-captured chunk per resident solver, each on its own stream, so
   requests that arrived at different times share the device;
3. retires finished requests: the final state is downloaded as the snapshot
   returned to the caller and the memory is released.

Latency of a request = completion time - arrival time.  The loop reports
p50 / p99 latency, queueing delay, aggregate grid-point-steps/s and
completed requests/s.  There is no reference counterpart (NLSEmagic
integrates one solve per call).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .api import Batch, Solver
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
    solo: bool = False
    snapshot: np.ndarray = field(repr=False, default=None)

    @property
    def latency(self):
        return self.done - self.arrival


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs, dtype=float), q)) if len(xs) else float("nan")


def summarize(done, wall, busy=None, launches=None, rejected=0):
    lat = [c.latency for c in done]
    qd = [c.admitted - c.arrival for c in done]
    pts = float(sum(c.points * c.steps for c in done))
    out = {
        "requests": len(done), "rejected": rejected, "wall_s": wall,
        "p50_latency_s": percentile(lat, 50), "p99_latency_s": percentile(lat, 99),
        "p50_queue_s": percentile(qd, 50), "p99_queue_s": percentile(qd, 99),
        "gpt_steps_per_s": pts / wall / 1e9 if wall else 0.0,
        "requests_per_s": len(done) / wall if wall else 0.0, "point_steps": pts,
    }
    if busy is not None:
        out["busy_s"] = busy
        out["gpt_steps_per_busy_s"] = pts / busy / 1e9 if busy else 0.0
    if launches is not None:
        out["launches"] = launches
    return out


class Server:
    def __init__(self, pool_bytes, chunk_steps=64, max_solves=8192, keep_snapshots=False,
                 solo_points=1 << 18, solo_bytes=None):
        self.batch = Batch(pool_bytes, max_solves)
        self.pool_bytes = int(pool_bytes)
        self.chunk_steps = int(chunk_steps)
        self.keep_snapshots = keep_snapshots
        self.solo_points = int(solo_points)
        self.solo_bytes = int(solo_bytes if solo_bytes is not None else pool_bytes)

    def close(self):
        self.batch.close()

    def is_solo(self, inst):
        return inst.U.ndim == 3 and inst.U.size >= self.solo_points

    def serve(self, requests, time_scale=1.0, max_wall=None):
        """Serve `requests` (objects with .rid, .arrival seconds, .inst with
        U, V, s, a, h, BC, method, k, steps, precision) in real time.
        Arrival times are multiplied by time_scale (0: all at once).  Returns
        a summary dict and the list of Completed records."""
        b = self.batch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting = deque()
        active = {}  # batch slot -> (request, admitted)
        solos = []   # [request, admitted, Solver, steps_left, bytes]
        solo_used = 0
        done = []
        rejected = []
        t0 = time.perf_counter()
        busy = 0.0
        launches = 0
        while pending or waiting or active or solos:
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                break
            while pending and pending[0].arrival * time_scale <= now:
                waiting.append(pending.popleft())
            # admission in arrival order, by the device-memory budgets
            while waiting:
                r = waiting[0]
                i = r.inst
                if self.is_solo(i):
                    need = Solver.bytes_for(i.U.shape, i.method, i.precision, i.BC)
                    if need > self.solo_bytes:
                        rejected.append(r.rid)
                        waiting.popleft()
                        continue
                    if solo_used + need > self.solo_bytes:
                        break  # wait for a resident solver to retire
                    sv = Solver(i.U.shape, method=i.method, precision=i.precision, BC=i.BC, s=i.s,
                                a=i.a, h2=i.h * i.h, k=i.k)
                    sv.upload(i.U, i.V)
                    solos.append([r, time.perf_counter() - t0, sv, int(i.steps), need])
                    solo_used += need
                    waiting.popleft()
                    continue
                need = Batch.bytes_for(i.U.shape, i.precision, i.method)
                if need > self.pool_bytes:
                    rejected.append(r.rid)
                    waiting.popleft()
                    continue
                try:
                    slot = b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, i.method,
                                 i.precision)
                except NLSEError as e:
                    if e.code == NLSE_ERR_CAPACITY:
                        break  # wait for pool memory to free up
                    raise
                active[slot] = (r, time.perf_counter() - t0)
                waiting.popleft()
            if not active and not solos:
                if pending:
                    dt = pending[0].arrival * time_scale - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                continue
            # one round: batched launch(es) plus a chunk of every resident solver
            ts = time.perf_counter()
            if active:
                b.run(self.chunk_steps)
            for sl in solos:
                n = min(self.chunk_steps, sl[3])
                sl[2].run(n)
                sl[3] -= n
                launches += n * sl[2].launches_per_step
            if active:
                b.sync()
                launches += b.last_launches
            for sl in solos:
                sl[2].sync()
            busy += time.perf_counter() - ts
            for slot in list(active):
                if b.remaining(slot) == 0:
                    r, tadm = active.pop(slot)
                    snap = b.download(slot)
                    done.append(Completed(r.rid, r.arrival * time_scale, tadm,
                                          time.perf_counter() - t0, int(r.inst.U.size),
                                          int(r.inst.steps), int(r.inst.precision), False,
                                          snap if self.keep_snapshots else None))
                    b.remove(slot)
            keep = []
            for sl in solos:
                if sl[3] > 0:
                    keep.append(sl)
                    continue
                r, tadm, sv, _, need = sl
                snap = sv.download()
                sv.close()
                solo_used -= need
                done.append(Completed(r.rid, r.arrival * time_scale, tadm,
                                      time.perf_counter() - t0, int(r.inst.U.size),
                                      int(r.inst.steps), int(r.inst.precision), True,
                                      snap if self.keep_snapshots else None))
            solos = keep
        wall = time.perf_counter() - t0
        return summarize(done, wall, busy, launches, len(rejected)), done


def serve_sequential(requests, time_scale=1.0, keep_snapshots=False):
    """Baseline: one solve at a time, first come first served, each through
    its own Solver (tiled 3D kernels, graph-captured chunks): create, upload,
    run all steps, download, release -- the reference's one-call-per-solve
    model without its per-call device reset.  The requests are run back to
    back; each one's latency is that of a single FIFO server fed by the same
    arrival times (start = max(previous finish, arrival))."""
    t0 = time.perf_counter()
    done = []
    clock = 0.0
    for r in sorted(requests, key=lambda r: r.arrival):
        i = r.inst
        arr = r.arrival * time_scale
        start = max(clock, arr)
        ts = time.perf_counter()
        s = Solver(i.U.shape, method=i.method, precision=i.precision, BC=i.BC, s=i.s, a=i.a,
                   h2=i.h * i.h, k=i.k)
        s.upload(i.U, i.V)
        s.run(i.steps)
        snap = s.download()
        s.close()
        clock = start + (time.perf_counter() - ts)
        done.append(Completed(r.rid, arr, start, clock, int(i.U.size), int(i.steps),
                              int(i.precision), True, snap if keep_snapshots else None))
    busy = time.perf_counter() - t0
    out = summarize(done, clock if clock > 0 else busy, busy)
    return out, done
