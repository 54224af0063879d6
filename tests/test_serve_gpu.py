"""Serving loop: continuous batching of a Poisson request stream.

Every request completes; each result is identical to the same solve run
alone (the batch never mixes solves), latency statistics are reported, and
admission honours the pool budget (requests wait, not fail, when it is full).
"""
import numpy as np
import pytest

from nlsemagic_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def small_stream(count=30, rate=400.0):
    return W.serving_requests(count=count, rate=rate, n1=(256, 2048), n2=(32, 96), n3=(12, 24),
                              steps=(20, 120))


def test_serving_results_equal_alone(gpu_lib):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.serve import Server, solve_flags
    reqs = small_stream()
    srv = Server(pool_bytes=1 << 28, chunk_steps=16, keep_snapshots=True)
    summary, done = srv.serve(reqs)
    srv.close()
    assert summary["requests"] == len(reqs)
    assert summary["p99_latency_s"] >= summary["p50_latency_s"] > 0
    by_id = {c.rid: c for c in done}
    for r in reqs[:12]:
        i = r.inst
        b = ng.Batch(1 << 26)
        sl = b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, i.method, i.precision,
                   flags=solve_flags(i, srv.fp64_fma))
        b.run(i.steps)
        assert bits_equal(by_id[r.rid].snapshot, b.download(sl))
        b.close()


def test_serving_waits_when_pool_is_full(gpu_lib):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.serve import Server
    reqs = small_stream(count=16, rate=1e6)  # all arrive at once
    biggest = max(ng.Batch.bytes_for(r.inst.U.shape, r.inst.precision) for r in reqs)
    srv = Server(pool_bytes=2 * biggest, chunk_steps=32)
    summary, done = srv.serve(reqs)
    srv.close()
    assert summary["requests"] == len(reqs)
    assert summary["rejected"] == 0
    assert summary["p99_queue_s"] > 0


def test_serving_solo_and_batched_results_equal_alone(gpu_lib):
    # 3D requests above solo_points run on their own resident solver (tiled
    # kernels), the rest in the batched launch; each result equals the same
    # solve run alone on the same path, bit for bit
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.serve import Server, serve_sequential, solve_flags
    reqs = W.serving_requests(count=24, rate=500.0, n1=(256, 1024), n2=(32, 64), n3=(18, 30),
                              steps=(20, 60))
    srv = Server(pool_bytes=1 << 28, chunk_steps=16, keep_snapshots=True, solo_points=8000)
    summary, done = srv.serve(reqs)
    srv.close()
    assert summary["requests"] == len(reqs)
    assert any(c.solo for c in done) and any(not c.solo for c in done)
    by_id = {r.rid: r for r in reqs}
    for c in done:
        i = by_id[c.rid].inst
        if c.solo:  # FP64 large solves take the contracted kernels
            want = ng.take_steps(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k,
                                 method=i.method, precision=i.precision,
                                 flags=solve_flags(i, srv.fp64_fma))
        else:  # small FP64 solves take the batch kernel's contracted copy
            b = ng.Batch(1 << 26)
            sl = b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, i.method, i.precision,
                       flags=solve_flags(i, srv.fp64_fma))
            b.run(i.steps)
            want = b.download(sl)
            b.close()
        assert bits_equal(c.snapshot, want)
    # the one-at-a-time baseline computes the same solves (single-solve path)
    seq, seq_done = serve_sequential(reqs[:6], keep_snapshots=True)
    for c in seq_done:
        i = by_id[c.rid].inst
        want = ng.take_steps(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, method=i.method,
                             precision=i.precision, flags=solve_flags(i, True))
        assert bits_equal(c.snapshot, want)


def test_serving_runs_least_remaining_work_first(gpu_lib):
    # large 3D requests queued together run one at a time (one per precision
    # class with per_class), the one with the least remaining work first, so
    # they complete in order of their work (within each class)
    from nlsemagic_gb300.serve import Server
    reqs = W.serving_requests(count=8, rate=1e3, ratio=(0, 0, 1), n3=(20, 28), steps=(20, 200))
    for per_class in (False, True):
        srv = Server(pool_bytes=1 << 28, chunk_steps=16, solo_points=1000, slice_s=1e-4,
                     per_class=per_class)
        summary, done = srv.serve(reqs, time_scale=0.0)
        srv.close()
        assert summary["requests"] == len(reqs) and all(c.solo for c in done)
        classes = (None,) if not per_class else sorted({r.inst.precision for r in reqs})
        for cls in classes:
            mine = [r for r in reqs if cls is None or r.inst.precision == cls]
            ids = {r.rid for r in mine}
            finished = [c.rid for c in sorted(done, key=lambda c: c.done) if c.rid in ids]
            assert finished == [r.rid for r in sorted(mine, key=lambda r: srv.work(r.inst))]
