"""Batched persistent launch: many uneven solves in one launch.

* FP64 solves in a batch are bit-identical to the C oracle; those added with
  NLSE_FLAG_FMA (contracted kernel copy) are within 1e-12 of it.
* A solve's result is identical alone and in a mixed batch (bitwise: solves
  never interact), and mixed-precision results are within the mixed
  tolerance of the FP64 oracle.
* Solves with different step counts each advance exactly their own count;
  chunked runs equal one long run; admission respects the pool budget.
"""
import numpy as np
import pytest

import oracle
from nlsemagic_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def smooth_case(ndim, n, method, BC, seed):
    rng = np.random.default_rng(seed)
    h = 0.3
    x = -n * h / 2 + h * np.arange(n)
    grids = np.meshgrid(*([x] * ndim), indexing="ij")
    r2 = sum(g * g for g in grids)
    c = rng.uniform(-1, 1, size=ndim)
    U = (np.exp(-r2 / (2 + 10 * rng.random())) * np.exp(1j * sum(ci * g for ci, g in zip(c, grids)))
         + 0.3).astype(complex)
    V = 0.5 * r2 / r2.max()
    s = float(rng.choice([-1.0, 1.0]))
    a = float(rng.uniform(0.5, 2.0))
    k = 0.6 * W.linear_stability_k(ndim, method, h, a)
    return dict(U=U if ndim > 1 else U.ravel(), V=V if ndim > 1 else V.ravel(), s=s, a=a, h2=h * h,
                BC=BC, k=k, method=method)


CASES = [(1, 300, 1, 2), (1, 257, 2, 1), (1, 1030, 2, 3), (2, 40, 1, 1), (2, 33, 2, 2),
         (2, 65, 2, 3), (3, 12, 1, 2), (3, 9, 2, 1), (1, 64, 1, 4), (1, 70, 2, 4)]


@pytest.fixture(scope="module")
def cases():
    return [smooth_case(*c, seed=10 + t) for t, c in enumerate(CASES)]


def oracle_run(c, steps, precision=2):
    return oracle.take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"],
                             method=c["method"], precision=precision, flags=oracle.MSD_GUARD)


def test_fp64_batch_bit_exact(gpu_lib, cases):
    import nlsemagic_gb300 as ng
    b = ng.Batch(1 << 28)
    steps = [13 + 3 * t for t in range(len(cases))]
    slots = [b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], st, c["k"], c["method"],
                   ng.PREC_DOUBLE) for c, st in zip(cases, steps)]
    b.run(max(steps))
    b.sync()
    assert b.last_launches == 1
    for c, st, sl in zip(cases, steps, slots):
        assert b.remaining(sl) == 0
        assert bits_equal(b.download(sl), oracle_run(c, st))
    b.close()


def test_mixed_batch_alone_equals_in_mix_and_tolerance(gpu_lib, cases):
    import nlsemagic_gb300 as ng
    steps = 40
    alone = []
    for c in cases:
        b = ng.Batch(1 << 26)
        sl = b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"], c["method"],
                   ng.PREC_MIXED)
        b.run(steps)
        alone.append(b.download(sl))
        b.close()
    b = ng.Batch(1 << 28)
    slots = []
    for t, c in enumerate(cases):
        # interleave FP64 solves into the mix
        slots.append(b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"],
                           c["method"], ng.PREC_MIXED))
        b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps + t, c["k"], c["method"],
              ng.PREC_DOUBLE)
    b.run(steps + len(cases))
    for c, a1, sl in zip(cases, alone, slots):
        mixed = b.download(sl)
        assert bits_equal(mixed, a1), "result differs alone vs in the mix"
        assert W.rel_l2(mixed, oracle_run(c, steps)) <= MIXED_TOL
    b.close()


def test_chunked_runs_equal_single_run(gpu_lib, cases):
    import nlsemagic_gb300 as ng
    c = cases[4]
    b1 = ng.Batch(1 << 26)
    s1 = b1.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 50, c["k"], c["method"],
                ng.PREC_MIXED)
    b1.run(50)
    b2 = ng.Batch(1 << 26)
    s2 = b2.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 50, c["k"], c["method"],
                ng.PREC_MIXED)
    for _ in range(7):
        b2.run(7)  # 49 steps
    assert b2.remaining(s2) == 1
    b2.run(7)
    assert b2.remaining(s2) == 0
    assert bits_equal(b1.download(s1), b2.download(s2))
    b1.close()
    b2.close()


def test_capacity_and_release(gpu_lib, cases):
    import nlsemagic_gb300 as ng
    c = cases[2]
    need = ng.Batch.bytes_for(c["U"].shape, ng.PREC_MIXED)
    b = ng.Batch(2 * need + 100, max_solves=8)
    s0 = b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 5, c["k"], c["method"],
               ng.PREC_MIXED)
    s1 = b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 5, c["k"], c["method"],
               ng.PREC_MIXED)
    with pytest.raises(ng.NLSEError) as ei:
        b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 5, c["k"], c["method"],
              ng.PREC_MIXED)
    assert ei.value.code == ng._lib.NLSE_ERR_CAPACITY
    assert b.stats()["active"] == 2
    b.remove(s0)
    s2 = b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 5, c["k"], c["method"],
               ng.PREC_MIXED)
    b.run(5)
    assert bits_equal(b.download(s1), b.download(s2))
    b.close()


def test_uneven_config4_sample(gpu_lib):
    # a slice of the uneven batch workload: every solve matches the FP64
    # oracle within the mixed tolerance after its steps
    import nlsemagic_gb300 as ng
    insts = W.batch_instances(count=24, steps=30, n1=(256, 2048), n2=(64, 128))
    b = ng.Batch(1 << 30)
    slots = [b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k, i.method, ng.PREC_MIXED)
             for i in insts]
    b.run(30)
    for i, sl in zip(insts, slots):
        want = oracle.take_steps(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, i.steps, i.k,
                                 method=i.method, precision=2, flags=oracle.MSD_GUARD)
        assert W.rel_l2(b.download(sl), want) <= MIXED_TOL
    b.close()


def test_mixed_batch_equals_single_solver(gpu_lib, cases):
    # 1D/2D: the batch evaluates every point with the same per-point
    # expressions as the single-solve path -- 1D segments and one-sided 1D
    # ends as the gather kernels (D staged in shared memory, or in scratch),
    # 2D rectangles as the single-pass 2D kernel (wide form with ghosts)
    # -- so the results are the same bits
    import nlsemagic_gb300 as ng
    steps = 17
    b = ng.Batch(1 << 28)
    picked = [c for c in cases if c["U"].ndim <= 2]
    slots = [b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"], c["method"],
                   ng.PREC_MIXED) for c in picked]
    b.run(steps)
    for c, sl in zip(picked, slots):
        one = ng.take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"],
                            method=c["method"], precision=ng.PREC_MIXED)
        assert bits_equal(b.download(sl), one)
        if c["U"].ndim == 1:  # the gather form too
            gat = ng.take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"],
                                method=c["method"], precision=ng.PREC_MIXED,
                                flags=ng.FLAG_MSD_GUARD | ng.FLAG_GATHER)
            assert bits_equal(b.download(sl), gat)
    b.close()


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
def test_mixed_batch_tile_edges(gpu_lib, method, BC):
    # sizes on every residue the batch's tiles treat differently: 1D
    # segments of 1024 (n = 1024 m + 1 shifts them by one point, n = 1024 m),
    # 2D rectangles of 32 x 16 (sides 32 m + 1, 16 m + 1, 32 m, thin grids);
    # each result is the single solver's, bit for bit
    import nlsemagic_gb300 as ng
    shapes = [(1025,), (2048,), (2049,), (3,), (1023,), (33, 17), (64, 48), (3, 97), (97, 3),
              (65, 49), (40, 33)]
    b = ng.Batch(1 << 28)
    picked, slots = [], []
    for t, shape in enumerate(shapes):
        c = smooth_case(len(shape), shape[0], method, BC, seed=500 + t)
        if len(shape) == 2:  # a non-square grid
            c2 = smooth_case(2, max(shape), method, BC, seed=600 + t)
            c["U"] = np.ascontiguousarray(c2["U"][:shape[0], :shape[1]])
            c["V"] = np.ascontiguousarray(c2["V"][:shape[0], :shape[1]])
        picked.append(c)
        slots.append(b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 9, c["k"],
                           c["method"], ng.PREC_MIXED))
    b.run(9)
    for c, sl in zip(picked, slots):
        one = ng.take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], 9, c["k"],
                            method=c["method"], precision=ng.PREC_MIXED)
        got = b.download(sl)
        assert np.all(np.isfinite(got))
        assert bits_equal(got, one), c["U"].shape
    b.close()


def test_batch_contracted_fp64_class(gpu_lib, cases):
    # FP64 solves added with NLSE_FLAG_FMA run on the contracted copy of the
    # batch kernel, a third launch beside the exact FP64 and mixed ones:
    # within 1e-12 of the oracle, each the same alone and in the mix, and the
    # exact FP64 solves of the same batch still bit-identical
    import nlsemagic_gb300 as ng
    fma = ng.FLAG_MSD_GUARD | ng.FLAG_FMA
    steps = 30
    alone = []
    for c in cases:
        b = ng.Batch(1 << 26)
        sl = b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps, c["k"], c["method"],
                   ng.PREC_DOUBLE, flags=fma)
        b.run(steps)
        alone.append(b.download(sl))
        b.close()
    b = ng.Batch(1 << 28)
    slots = []
    for c in cases:
        slots.append(("fma", b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps,
                                   c["k"], c["method"], ng.PREC_DOUBLE, flags=fma)))
        slots.append(("exact", b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps,
                                     c["k"], c["method"], ng.PREC_DOUBLE)))
        slots.append(("mixed", b.add(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], steps,
                                     c["k"], c["method"], ng.PREC_MIXED)))
    b.run(steps)
    b.sync()
    assert b.last_launches == 3
    for t, c in enumerate(cases):
        ref = oracle_run(c, steps)
        got = {kind: b.download(sl) for kind, sl in slots[3 * t:3 * t + 3]}
        assert bits_equal(got["exact"], ref)
        assert bits_equal(got["fma"], alone[t])
        err = np.linalg.norm((got["fma"] - ref).ravel()) / np.linalg.norm(ref.ravel())
        assert err <= 1e-12, err
        err = np.linalg.norm((got["mixed"] - ref).ravel()) / np.linalg.norm(ref.ravel())
        assert err <= MIXED_TOL, err
    b.close()


def test_batch_rejects_contracted_mixed(gpu_lib):
    # NLSE_FLAG_FMA selects a form of the FP64 class only
    import nlsemagic_gb300 as ng
    U = np.ones(64, complex)
    b = ng.Batch(1 << 24)
    try:
        with pytest.raises(ng.NLSEError) as e:
            b.add(U, np.zeros(64), -1.0, 1.0, 0.01, 1, 4, 1e-3, 1, ng.PREC_MIXED,
                  flags=ng.FLAG_MSD_GUARD | ng.FLAG_FMA)
        assert e.value.code == ng._lib.NLSE_ERR_ARG
    finally:
        b.close()
