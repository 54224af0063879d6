"""Exact-precision 2D stage kernels.  FP32 takes the single-pass tile kernel
(the stage input staged per tile in shared memory, 2SHOC's D formed there,
one launch per stage); FP64 keeps the gather kernels.  Every
combination is bit-identical to the oracle (the reference C integrators'
arithmetic) for both precisions, both methods, every boundary code and
every tile-height setting, on grids whose sides fall on every residue the
tiling treats differently (n = 32 m + 1 and TY m + 1 shift the tiles by one
cell; n = 32 m; thin and tiny grids); and with the knob off, the gather
kernels give the same bits."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(3, 3), (4, 5), (3, 40), (40, 3), (33, 33), (32, 64), (65, 31), (97, 34),
          (70, 129), (100, 66), (2 * 32 + 2, 5 * 32 + 1), (17, 9)]


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    U = (0.9 + 0.1 * rng.standard_normal(shape)) + 0.1j * rng.standard_normal(shape)
    V = 0.05 * rng.random(shape)
    return U, V


def _gpu(U, V, BC, method, prec, steps, ty=0, wide2d=1):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    old = {key: autotune.get_knob(key) for key in ("wide2d", "wide2d.ty")}
    try:
        autotune.set_knob("wide2d", wide2d)
        autotune.set_knob("wide2d.ty", ty)
        return ng.take_steps(U, V, -1.0, 0.9, 0.09, BC, steps, 0.002, method=method,
                             precision=prec, flags=ng.FLAG_MSD_GUARD)
    finally:
        for key, v in old.items():
            autotune.set_knob(key, v)


@pytest.mark.parametrize("prec", [2, 1])
@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("shape", SHAPES)
def test_tile2d_bit_exact(gpu_lib, shape, method, BC, prec):
    U, V = _case(shape, sum(shape) + 10 * method + BC + 100 * prec)
    steps = 4
    want = oracle.take_steps(U, V, -1.0, 0.9, 0.09, BC, steps, 0.002, method=method,
                             precision=prec, flags=oracle.MSD_GUARD)
    for ty in (0, 8, 16, 32):
        assert bits_equal(_gpu(U, V, BC, method, prec, steps, ty=ty), want), ty


@pytest.mark.parametrize("prec", [2, 1])
def test_tile2d_knob_off_same_bits(gpu_lib, prec):
    U, V = _case((45, 38), 5)
    on = _gpu(U, V, 2, 2, prec, 6)
    off = _gpu(U, V, 2, 2, prec, 6, wide2d=0)
    assert bits_equal(on, off)


def test_tile2d_launches_per_step(gpu_lib):
    # 2SHOC: one launch per stage in FP32 and mixed, D then F in FP64
    import nlsemagic_gb300 as ng
    for prec, want in ((1, 4), (2, 8), (3, 4)):
        with ng.Solver((64, 48), method=2, precision=prec, BC=1, s=-1.0, a=1.0, h2=0.09,
                       k=0.002) as sv:
            assert sv.launches_per_step == want


@pytest.mark.parametrize("shape", [(3, 700000), (700000, 3)])
def test_tile2d_tall_grid(gpu_lib, shape):
    # more tile rows than a launch's gridDim.y allows: bit-exact all the same
    U, V = _case(shape, 77)
    want = oracle.take_steps(U, V, -1.0, 0.9, 0.09, 1, 2, 0.002, method=2, precision=1,
                             flags=oracle.MSD_GUARD)
    assert bits_equal(_gpu(U, V, 1, 2, 1, 2, ty=8), want)
