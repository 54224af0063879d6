"""Parity at the full sizes of the benchmark configurations, against the C oracle.

The unit tests elsewhere pin every kernel on small and edge grids; here the
whole runs of the configurations are compared end to end:

* configuration 2 -- 2D 2SHOC, 512^2 dark vortices, Dirichlet, all 2000 RK4
  steps: FP64 bit-identical to the FP64 oracle, FP32 bit-identical to the
  FP32 oracle, mixed within 1e-6 relative L2 of the FP64 oracle; the mass
  sum |U|^2 h^2 of the FP64 result equal to the oracle's;
* configuration 3 -- 3D, 320^3 vortex rings in a harmonic trap, MSD: 2SHOC
  for all 500 RK4 steps, CD for 100; FP64 bit-identical, mixed within 1e-6;
* on both, the FP64 class's contracted form (NLSE_FLAG_FMA) within 1e-12.

The oracle (test infrastructure, oracle/) runs each solve over all host cores
(oracle.set_threads, same bits as serial).  Its runs are queued on a
background thread when the module starts, so they overlap the GPU work;
each test waits for the result it needs.  The loops follow
src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_2SHOC.c:369-380 and
src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC.c:507-521.
"""
import os
import threading
from concurrent.futures import Future

import numpy as np
import pytest

import oracle
from nlsemagic_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6  # relative L2 against the FP64 oracle
C3_CD_STEPS = 100


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def mass(U, h, ndim):
    return float(np.sum(np.abs(U) ** 2)) * h ** ndim


class OracleQueue:
    """Oracle runs in order on one background thread, each over all cores."""

    def __init__(self, jobs):
        self.futures = {name: Future() for name, _ in jobs}
        self.jobs = jobs
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _run(self):
        oracle.set_threads(os.cpu_count() or 1)
        try:
            for name, fn in self.jobs:
                try:
                    self.futures[name].set_result(fn())
                except Exception as e:  # surfaced by the test that waits
                    self.futures[name].set_exception(e)
        finally:
            oracle.set_threads(1)

    def get(self, name):
        return self.futures[name].result()


@pytest.fixture(scope="module")
def work(gpu_lib):
    w2 = W.dark_vortices_2d()
    w3 = W.vortex_rings_3d()
    w3cd = W.vortex_rings_3d(method=1)

    def orc(w, steps, precision):
        return lambda: oracle.take_steps(w.U, w.V, w.s, w.a, w.h2, w.BC, steps, w.k,
                                         method=w.method, precision=precision,
                                         flags=oracle.MSD_GUARD)

    q = OracleQueue([("c2_fp64", orc(w2, w2.steps, 2)), ("c2_fp32", orc(w2, w2.steps, 1)),
                     ("c3cd_fp64", orc(w3cd, C3_CD_STEPS, 2)),
                     ("c3_fp64", orc(w3, w3.steps, 2))])
    yield {"w2": w2, "w3": w3, "w3cd": w3cd, "oracle": q}
    q.t.join()


def gpu_run(w, steps, precision, flags=None):
    import nlsemagic_gb300 as ng
    if flags is None:
        flags = ng.FLAG_MSD_GUARD
    with ng.Solver(w.U.shape, method=w.method, precision=precision, BC=w.BC, s=w.s, a=w.a,
                   h2=w.h2, k=w.k, flags=flags) as sv:
        sv.upload(w.U, w.V)
        sv.run(steps)
        sv.sync()
        return sv.download()


def test_config2_fp64_full_run_bit_exact(work):
    import nlsemagic_gb300 as ng
    w = work["w2"]
    got = gpu_run(w, w.steps, ng.PREC_DOUBLE)
    ref = work["oracle"].get("c2_fp64")
    assert bits_equal(got, ref)
    assert W.rel_l2(got, ref) <= 1e-12
    assert mass(got, w.h, 2) == mass(ref, w.h, 2)


def test_config2_fp32_full_run_bit_exact(work):
    import nlsemagic_gb300 as ng
    w = work["w2"]
    got = gpu_run(w, w.steps, ng.PREC_SINGLE)
    assert bits_equal(got, work["oracle"].get("c2_fp32"))


def test_config2_mixed_full_run_within_tolerance(work):
    import nlsemagic_gb300 as ng
    w = work["w2"]
    got = gpu_run(w, w.steps, ng.PREC_MIXED)
    ref = work["oracle"].get("c2_fp64")
    err = W.rel_l2(got, ref)
    assert err <= MIXED_TOL, err
    m0 = mass(w.U, w.h, 2)
    assert abs(mass(got, w.h, 2) - mass(ref, w.h, 2)) <= 1e-6 * m0


def test_config3_cd_320_bit_exact_and_mixed(work):
    import nlsemagic_gb300 as ng
    w = work["w3cd"]
    got = gpu_run(w, C3_CD_STEPS, ng.PREC_DOUBLE)
    mixed = gpu_run(w, C3_CD_STEPS, ng.PREC_MIXED)
    ref = work["oracle"].get("c3cd_fp64")
    assert bits_equal(got, ref)
    err = W.rel_l2(mixed, ref)
    assert err <= MIXED_TOL, err


def test_config3_2shoc_320_full_run(work):
    import nlsemagic_gb300 as ng
    w = work["w3"]
    got = gpu_run(w, w.steps, ng.PREC_DOUBLE)
    mixed = gpu_run(w, w.steps, ng.PREC_MIXED)
    ref = work["oracle"].get("c3_fp64")
    assert bits_equal(got, ref)
    assert W.rel_l2(got, ref) <= 1e-12
    err = W.rel_l2(mixed, ref)
    assert err <= MIXED_TOL, err
    m0 = mass(w.U, w.h, 3)
    assert mass(got, w.h, 3) == mass(ref, w.h, 3)
    assert abs(mass(mixed, w.h, 3) - mass(ref, w.h, 3)) <= 1e-6 * m0


def test_fp64_contracted_full_runs_within_1e12(work):
    import nlsemagic_gb300 as ng
    flags = ng.FLAG_MSD_GUARD | ng.FLAG_FMA
    for w, name in ((work["w2"], "c2_fp64"), (work["w3"], "c3_fp64")):
        got = gpu_run(w, w.steps, ng.PREC_DOUBLE, flags)
        ref = work["oracle"].get(name)
        err = W.rel_l2(got, ref)
        assert err <= 1e-12, (w.name, err)
