"""Mixed-precision 2D single-pass stage kernel (one launch per RK4 stage, the
2SHOC wide form with ghost cells beyond the faces, face points in the same
launch).  Against the FP64 oracle within the mixed tolerance on grids whose
sides fall on every residue the tiling treats differently (n = 32 m + 1,
which shifts the tiles by one cell; n = 32 m; thin and tiny grids), for
both methods, every boundary code and every tile height; the same bits run
after run; and within the tolerance of the gather form it replaces."""
import numpy as np
import pytest

from nlsemagic_gb300 import workloads as W
import oracle

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6  # relative L2 vs the FP64 oracle

SHAPES = [(3, 3), (4, 5), (3, 40), (40, 3), (33, 33), (32, 64), (65, 31), (97, 34),
          (70, 129), (100, 66), (2 * 32 + 2, 5 * 32 + 1)]


def _field(shape):
    h = 0.3
    axes = [-n * h / 2 + h * np.arange(n) for n in shape]
    X, Y = np.meshgrid(*axes, indexing="ij")
    r2 = X * X + Y * Y
    U = (np.exp(-r2 / 20.0) * np.exp(0.3j * X + 0.1j * Y) + 0.4).astype(complex)
    V = 0.3 * r2 / max(r2.max(), 1e-30)
    return U, V, h


def _gpu(U, V, h, BC, method, steps, k, wide2d=1, gather=False, ty=0):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    old = {key: autotune.get_knob(key) for key in ("wide2d", "wide2d.ty")}
    try:
        autotune.set_knob("wide2d", wide2d)
        autotune.set_knob("wide2d.ty", ty)
        flags = ng.FLAG_MSD_GUARD | (ng.FLAG_GATHER if gather else 0)
        return np.ascontiguousarray(
            ng.take_steps(U, V, -1.0, 1.0, h * h, BC, steps, k, method=method,
                          precision=ng.PREC_MIXED, flags=flags))
    finally:
        for key, v in old.items():
            autotune.set_knob(key, v)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
def test_wide2d_against_oracle(gpu_lib, shape, method, BC):
    U, V, h = _field(shape)
    k = 0.5 * W.linear_stability_k(2, method, h, 1.0)
    steps = 12
    want = oracle.take_steps(U, V, -1.0, 1.0, h * h, BC, steps, k, method=method, precision=2,
                             flags=oracle.MSD_GUARD)
    for ty in (0, 8, 16, 32):  # by grid size, then each tile height
        got = _gpu(U, V, h, BC, method, steps, k, ty=ty)
        assert np.all(np.isfinite(got))
        assert W.rel_l2(got, want) <= MIXED_TOL, ty
    # the gather form it replaces: same tolerance against the oracle
    assert W.rel_l2(_gpu(U, V, h, BC, method, steps, k, wide2d=0), want) <= MIXED_TOL


@pytest.mark.parametrize("ty", [8, 16, 32])
@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
def test_wide2d_deterministic(gpu_lib, method, BC, ty):
    U, V, h = _field((161, 96))
    k = 0.5 * W.linear_stability_k(2, method, h, 1.0)
    first = _gpu(U, V, h, BC, method, 40, k, ty=ty)
    for _ in range(2):
        again = _gpu(U, V, h, BC, method, 40, k, ty=ty)
        assert np.array_equal(again.view(np.float64), first.view(np.float64))


def test_wide2d_knob_off_is_the_gather_form(gpu_lib):
    # with the knob off the tiled solver takes the gather kernels: the same
    # bits as the solver created with the gather flag
    U, V, h = _field((45, 38))
    k = 0.5 * W.linear_stability_k(2, 2, h, 1.0)
    off = _gpu(U, V, h, 2, 2, 9, k, wide2d=0)
    gat = _gpu(U, V, h, 2, 2, 9, k, wide2d=1, gather=True)
    assert np.array_equal(off.view(np.float64), gat.view(np.float64))


def test_wide2d_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("wide2d", 2)
    with pytest.raises(Exception):
        autotune.set_knob("wide2d.ty", 4)


@pytest.mark.parametrize("shape", [(3, 700000), (700000, 3)])
def test_wide2d_tall_grid(gpu_lib, shape):
    # more tile rows than a launch's gridDim.y allows (65535): tiles are
    # numbered in a one-dimensional grid
    U, V, h = _field(shape)
    k = 0.5 * W.linear_stability_k(2, 2, h, 1.0)
    want = oracle.take_steps(U, V, -1.0, 1.0, h * h, 2, 3, k, method=2, precision=2,
                             flags=oracle.MSD_GUARD)
    for ty in (0, 8):
        got = _gpu(U, V, h, 2, 2, 3, k, ty=ty)
        assert W.rel_l2(got, want) <= MIXED_TOL
