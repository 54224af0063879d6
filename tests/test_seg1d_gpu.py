"""1D staged-segment stage kernels: the stage input staged per segment of
256 points in shared memory, 2SHOC's D formed there, one launch per stage.
The same bits as the gather kernels for every precision class, both methods
and every boundary code they serve (1-3), on sizes at every residue the
segments treat differently (n = 256 m + 1 shifts them by one point; n =
256 m; tiny grids); FP64 and FP32 bit-identical to the oracle, mixed within
its tolerance; one launch per stage."""
import numpy as np
import pytest

import oracle
from nlsemagic_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
SIZES = [3, 4, 255, 256, 257, 513, 1000, 2049, 2050, 4097, 5000, 65537]


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def _case(n):
    h = 0.1
    x = -n * h / 2 + h * np.arange(n)
    U = (np.exp(-x * x / 40.0) * np.exp(0.4j * x) + 0.3).astype(complex)
    V = 0.2 * x * x / max((x * x).max(), 1e-30)
    return U, V, h


def _run(U, V, h, BC, method, steps, k, gather=False, seg=1, prec=3):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    old = {key: autotune.get_knob(key) for key in ("seg1d", "small1d.max_points")}
    try:
        autotune.set_knob("seg1d", seg)
        autotune.set_knob("small1d.max_points", 0)  # every size through the stage kernels
        flags = ng.FLAG_MSD_GUARD | (ng.FLAG_GATHER if gather else 0)
        return ng.take_steps(U, V, -1.0, 1.0, h * h, BC, steps, k, method=method,
                             precision=prec, flags=flags)
    finally:
        for key, v in old.items():
            autotune.set_knob(key, v)


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("n", SIZES)
def test_seg1d_same_bits_as_gather(gpu_lib, n, method, BC):
    U, V, h = _case(n)
    k = 0.5 * W.linear_stability_k(1, method, h, 1.0)
    got = _run(U, V, h, BC, method, 11, k)
    assert np.all(np.isfinite(got))
    assert bits_equal(got, _run(U, V, h, BC, method, 11, k, gather=True))
    assert bits_equal(got, _run(U, V, h, BC, method, 11, k, seg=0))
    if n <= 5000:
        want = oracle.take_steps(U, V, -1.0, 1.0, h * h, BC, 11, k, method=method, precision=2,
                                 flags=oracle.MSD_GUARD)
        assert W.rel_l2(got, want) <= MIXED_TOL


@pytest.mark.parametrize("prec", [2, 1])
@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("n", SIZES)
def test_seg1d_exact_bit_exact(gpu_lib, n, method, BC, prec):
    U, V, h = _case(n)
    k = 0.5 * W.linear_stability_k(1, method, h, 1.0)
    got = _run(U, V, h, BC, method, 7, k, prec=prec)
    assert bits_equal(got, _run(U, V, h, BC, method, 7, k, gather=True, prec=prec))
    if n <= 5000:
        want = oracle.take_steps(U, V, -1.0, 1.0, h * h, BC, 7, k, method=method, precision=prec,
                                 flags=oracle.MSD_GUARD)
        assert bits_equal(got, want)


def test_seg1d_launches_per_step(gpu_lib):
    import nlsemagic_gb300 as ng
    for prec in (1, 2, 3):
        with ng.Solver((5000,), method=2, precision=prec, BC=2, s=-1.0, a=1.0, h2=0.01,
                       k=1e-3) as sv:
            assert sv.launches_per_step == 4


def test_seg1d_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("seg1d", 3)
