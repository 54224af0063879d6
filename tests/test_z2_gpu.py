"""Mixed-precision 3D interior kernel, two planes per iteration: the same
bits as the one-plane kernel (same per-point arithmetic), run after run, for
both methods and every boundary condition, on grids and z chunks with odd
and even plane counts (the last iteration of a chunk may hold a single
plane), at each of its tile heights (32 x 4, 32 x 8, 32 x 16)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [((19, 17, 20), 0), ((21, 12, 34), 0), ((40, 40, 40), 0), ((3, 3, 4), 0),
         ((70, 45, 100), 0), ((37, 33, 66), 5), ((37, 33, 66), 7), ((50, 24, 32), 16)]


def _run(shape, BC, z2, zc, steps=3, method=2, ty=8):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    z, y, x = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    U = (0.8 + 0.2 * np.cos(2.1 * x + 0.3) * np.cos(1.7 * y) * np.cos(1.3 * z + 0.5)
         + 0.15j * np.sin(1.9 * x + 1.1 * y + 0.7 * z))
    V = 0.5 + 0.5 * (x - 0.5) ** 2 + 0.3 * (y - 0.4) ** 2 + 0.2 * z
    old = {k: autotune.get_knob(k) for k in ("wide.z2", "wide.zc", "wide.ty")}
    try:
        autotune.set_knob("wide.z2", z2)
        autotune.set_knob("wide.zc", zc)
        autotune.set_knob("wide.ty", ty)
        with ng.Solver(shape, method=method, precision=ng.PREC_MIXED, BC=BC, s=-1.0, a=1.0,
                       h2=0.09, k=0.004) as sv:
            sv.upload(U, V)
            sv.run(steps)
            return np.ascontiguousarray(sv.download())
    finally:
        for k, v in old.items():
            autotune.set_knob(k, v)


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("shape,zc", CASES)
def test_two_planes_match_one(gpu_lib, shape, zc, BC, method):
    one = _run(shape, BC, 0, zc, method=method)
    assert np.all(np.isfinite(one))
    for _ in range(2):
        two = _run(shape, BC, 1, zc, method=method)
        assert np.array_equal(two.view(np.float64), one.view(np.float64)), \
            "max |diff| %g" % np.max(np.abs(two - one))


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("shape,zc", [((19, 17, 20), 0), ((37, 33, 66), 5), ((70, 45, 100), 0),
                                      ((36, 9, 12), 0)])
def test_tile_heights_give_the_same_bits(gpu_lib, shape, zc, BC, method):
    ref = _run(shape, BC, 1, zc, method=method, ty=8)
    for ty in (4, 16):
        got = _run(shape, BC, 1, zc, method=method, ty=ty)
        assert np.array_equal(got.view(np.float64), ref.view(np.float64)), \
            "tile height %d: max |diff| %g" % (ty, np.max(np.abs(got - ref)))
