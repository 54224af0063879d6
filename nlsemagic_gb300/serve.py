"""Continuous-batching request loop.

Requests (solves with their own dimension, grid, step count and precision
class) arrive over time.  The loop keeps the device busy with two kinds of
work in flight at once, each on its own stream, and polls them without
blocking:

1. **The batch.**  Small solves (1D, 2D, and 3D below ``solo_points``) take
   a slot in the batched persistent launch (:class:`~nlsemagic_gb300.api.Batch`,
   admitted by its pool budget while no launch is in flight).  Each launch
   advances every admitted solve by up to ``chunk_steps`` RK4 steps; a new
   launch starts as soon as the previous one finishes, so requests that
   arrive meanwhile join at the next launch.
2. **One large solve per precision class.**  Large 3D solves get a resident
   :class:`~nlsemagic_gb300.api.Solver` (the tiled 3D stage kernels),
   admitted against ``solo_bytes``.  One of each class runs at a time, a
   slice of about ``slice_s`` seconds of estimated work; at every slice
   boundary the admitted large solve of that class with the least remaining
   work goes next (shortest remaining processing time), so a short request
   is never stuck behind a long one, and a long one does not share the GPU
   with others of its kind.  The two classes run side by side because they
   load different units: an FP64 solve is bound by FP64 issue with DRAM
   nearly idle, a mixed solve by HBM bandwidth (``per_class=False``: one
   large solve at a time).

With ``fp64_fma`` (default) the FP64 solves run the contracted FP64
kernels (NLSE_FLAG_FMA): the large ones on their solver, the small ones in
the batched launch's contracted FP64 class.

Work is estimated as points x steps, times ``fp64_cost`` for the FP64 class
(about its speed ratio to the mixed class).  Waiting requests are admitted
least work first (``order="srpt"``) or in arrival order
(``order="fifo"``).  State and potential are uploaded once and stay resident
until the request completes; the final state is downloaded as the snapshot
returned to the caller.

Latency of a request = completion time - arrival time.  The loop reports
p50 / p99 latency, queueing delay, aggregate grid-point-steps/s and
completed requests/s.  There is no reference counterpart (NLSEmagic
integrates one solve per call; its drivers loop over chunks of one solve,
src/NLSEmagic3D/NLSEmagic3D.m:298-344).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .api import Batch, Solver
from ._lib import (FLAG_FMA, FLAG_MSD_GUARD, NLSE_ERR_CAPACITY, PREC_DOUBLE,
                   NLSEError)


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


def solve_flags(inst, fp64_fma):
    """Problem flags of a request, on its own Solver or in the batch: the MSD
    guard, and for FP64 requests with fp64_fma the contracted FP64 kernels
    (NLSE_FLAG_FMA: within 1e-12 of the reference's bits, fewer FP64
    instructions)."""
    fma = fp64_fma and inst.precision == PREC_DOUBLE
    return FLAG_MSD_GUARD | (FLAG_FMA if fma else 0)


class _Solo:
    __slots__ = ("req", "admitted", "solver", "left", "bytes", "inflight")

    def __init__(self, req, admitted, solver, left, nbytes):
        self.req, self.admitted, self.solver = req, admitted, solver
        self.left, self.bytes, self.inflight = left, nbytes, 0


class Server:
    def __init__(self, pool_bytes, chunk_steps=64, max_solves=8192, keep_snapshots=False,
                 solo_points=1 << 18, solo_bytes=None, order="srpt", slice_s=0.02,
                 fp64_cost=12.0, mixed_rate=15e9, per_class=True, fp64_fma=True):
        if order not in ("srpt", "fifo"):
            raise ValueError("order must be 'srpt' or 'fifo'")
        self.batch = Batch(pool_bytes, max_solves)
        self.pool_bytes = int(pool_bytes)
        self.chunk_steps = int(chunk_steps)
        self.keep_snapshots = keep_snapshots
        self.solo_points = int(solo_points)
        self.solo_bytes = int(solo_bytes if solo_bytes is not None else pool_bytes)
        self.order = order
        self.slice_s = float(slice_s)
        self.fp64_cost = float(fp64_cost)
        self.mixed_rate = float(mixed_rate)
        self.per_class = bool(per_class)
        self.fp64_fma = bool(fp64_fma)

    def close(self):
        self.batch.close()

    def is_solo(self, inst):
        return inst.U.ndim == 3 and inst.U.size >= self.solo_points

    def work(self, inst, steps=None):
        """Estimated work: point-steps, FP64 weighted by fp64_cost."""
        w = float(inst.U.size) * (inst.steps if steps is None else steps)
        return w * (self.fp64_cost if inst.precision == PREC_DOUBLE else 1.0)

    def _slice_steps(self, solo):
        # steps of about slice_s seconds at the estimated rate
        per_step = self.work(solo.req.inst, 1) / self.mixed_rate
        n = max(1, int(self.slice_s / per_step)) if per_step > 0 else solo.left
        return min(solo.left, n)

    def _classes(self, solos):
        """Running slots for large solves: one per precision class present
        (per_class), or a single shared one."""
        if not self.per_class:
            return [0] if solos else []
        return sorted({x.req.inst.precision for x in solos})

    def _key(self, r):
        return self.work(r.inst) if self.order == "srpt" else r.arrival

    def serve(self, requests, time_scale=1.0, max_wall=None):
        """Serve `requests` (objects with .rid, .arrival seconds, .inst with
        U, V, s, a, h, BC, method, k, steps, precision) in real time.
        Arrival times are multiplied by time_scale (0: all at once).  Returns
        a summary dict and the list of Completed records."""
        b = self.batch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        wait_small, wait_solo = [], []
        active = {}  # batch slot -> (request, admitted)
        solos = []   # admitted large solves
        running = {}  # precision class -> the large solve of it with a slice in flight
        batch_busy = False
        solo_used = 0
        done, rejected = [], []
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        busy, busy_since, launches = 0.0, None, 0

        def finish(r, tadm, snap, solo):
            done.append(Completed(r.rid, r.arrival * time_scale, tadm, clock(),
                                  int(r.inst.U.size), int(r.inst.steps), int(r.inst.precision),
                                  solo, snap if self.keep_snapshots else None))

        while pending or wait_small or wait_solo or active or solos:
            now = clock()
            if max_wall is not None and now > max_wall:
                break
            while pending and pending[0].arrival * time_scale <= now:
                r = pending.popleft()
                (wait_solo if self.is_solo(r.inst) else wait_small).append(r)
            progressed = False
            # ---- admission (the batch only between its launches)
            if wait_small and not batch_busy:
                wait_small.sort(key=self._key)
                keep = []
                for r in wait_small:
                    i = r.inst
                    if Batch.bytes_for(i.U.shape, i.precision, i.method) > self.pool_bytes:
                        rejected.append(r.rid)
                        continue
                    try:
                        slot = b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, i.method,
                                     i.precision, flags=solve_flags(i, self.fp64_fma))
                    except NLSEError as e:
                        if e.code != NLSE_ERR_CAPACITY:
                            raise
                        keep.append(r)  # waits for pool memory
                        continue
                    active[slot] = (r, clock())
                wait_small = keep
            if wait_solo:
                wait_solo.sort(key=self._key)
                keep = []
                for r in wait_solo:
                    i = r.inst
                    need = Solver.bytes_for(i.U.shape, i.method, i.precision, i.BC)
                    if need > self.solo_bytes:
                        rejected.append(r.rid)
                        continue
                    if solo_used + need > self.solo_bytes:
                        keep.append(r)  # waits for a large solve to retire
                        continue
                    sv = Solver(i.U.shape, method=i.method, precision=i.precision, BC=i.BC, s=i.s,
                                a=i.a, h2=i.h * i.h, k=i.k, flags=solve_flags(i, self.fp64_fma))
                    sv.upload(i.U, i.V)
                    solos.append(_Solo(r, clock(), sv, int(i.steps), need))
                    solo_used += need
                wait_solo = keep
            # ---- launches
            if not batch_busy and active:
                b.run(self.chunk_steps)
                batch_busy = True
                progressed = True
            for cls in self._classes(solos):
                if cls in running:
                    continue
                mine = [x for x in solos if x.req.inst.precision == cls or not self.per_class]
                if not mine:
                    continue
                x = min(mine, key=lambda x: (self.work(x.req.inst, x.left)
                                             if self.order == "srpt" else x.req.arrival))
                n = self._slice_steps(x)
                x.solver.run(n)
                x.inflight = n
                running[cls] = x
                launches += n * x.solver.launches_per_step
                progressed = True
            if (batch_busy or running) and busy_since is None:
                busy_since = clock()
            # ---- completions
            if batch_busy and b.idle():
                batch_busy = False
                launches += b.last_launches
                for slot in list(active):
                    if b.remaining(slot) == 0:
                        r, tadm = active.pop(slot)
                        snap = b.download(slot)
                        b.remove(slot)
                        finish(r, tadm, snap, False)
                progressed = True
            for cls, x in list(running.items()):
                if not x.solver.idle():
                    continue
                x.left -= x.inflight
                x.inflight = 0
                if x.left <= 0:
                    snap = x.solver.download()
                    x.solver.close()
                    solo_used -= x.bytes
                    solos.remove(x)
                    finish(x.req, x.admitted, snap, True)
                del running[cls]
                progressed = True
            if not batch_busy and not running and busy_since is not None:
                busy += clock() - busy_since
                busy_since = None
            if progressed:
                continue
            if batch_busy or running:
                time.sleep(0.0002)  # work in flight: poll again shortly
            elif pending and not wait_small and not wait_solo:
                dt = pending[0].arrival * time_scale - clock()
                if dt > 0:
                    time.sleep(dt)
        if busy_since is not None:
            busy += clock() - busy_since
        wall = clock()
        return summarize(done, wall, busy, launches, len(rejected)), done


def serve_sequential(requests, time_scale=1.0, keep_snapshots=False, fp64_fma=True):
    """Baseline: one solve at a time, first come first served, each through
    its own Solver (tiled 3D kernels, graph-captured chunks): create, upload,
    run all steps, download, release -- the reference's one-call-per-solve
    model without its per-call device reset.  The requests are run back to
    back; each one's latency is that of a single FIFO server fed by the same
    arrival times (start = max(previous finish, arrival)).  FP64 requests take
    the same arithmetic as the server's large solves (solve_flags)."""
    t0 = time.perf_counter()
    done = []
    clock = 0.0
    for r in sorted(requests, key=lambda r: r.arrival):
        i = r.inst
        arr = r.arrival * time_scale
        start = max(clock, arr)
        ts = time.perf_counter()
        s = Solver(i.U.shape, method=i.method, precision=i.precision, BC=i.BC, s=i.s, a=i.a,
                   h2=i.h * i.h, k=i.k, flags=solve_flags(i, fp64_fma))
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
