"""Mixed-precision 3D 2SHOC with programmatic dependent launch: a stage's
interior tiles start while the face kernels of the stage before still run.
The results must not depend on that overlap: bit-identical to plain stream
order, run after run, for every boundary condition and on grids whose tiles
are all at a face (no interior tile) or mostly interior."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(19, 17, 20), (21, 12, 33), (40, 40, 40), (3, 3, 3), (70, 45, 100), (96, 64, 130)]


def _run(shape, BC, pdl, steps=3):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    z, y, x = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    U = (0.8 + 0.2 * np.cos(2.1 * x + 0.3) * np.cos(1.7 * y) * np.cos(1.3 * z + 0.5)
         + 0.15j * np.sin(1.9 * x + 1.1 * y + 0.7 * z))
    V = 0.5 + 0.5 * (x - 0.5) ** 2 + 0.3 * (y - 0.4) ** 2 + 0.2 * z
    old = autotune.get_knob("wide.pdl")
    try:
        autotune.set_knob("wide.pdl", pdl)
        with ng.Solver(shape, method=2, precision=ng.PREC_MIXED, BC=BC, s=-1.0, a=1.0,
                       h2=0.09, k=0.004) as sv:
            sv.upload(U, V)
            sv.run(steps)
            return np.ascontiguousarray(sv.download())
    finally:
        autotune.set_knob("wide.pdl", old)


@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("shape", SHAPES)
def test_pdl_matches_stream_order(gpu_lib, shape, BC):
    plain = _run(shape, BC, 0)
    assert np.all(np.isfinite(plain))
    for _ in range(2):
        over = _run(shape, BC, 1)
        assert np.array_equal(over.view(np.float64), plain.view(np.float64)), \
            "max |diff| %g" % np.max(np.abs(over - plain))


def test_pdl_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("wide.pdl", 2)
