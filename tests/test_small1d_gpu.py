"""Small FP32 and mixed 1D solves run each chunk in one single-block launch
(every pass of every RK4 step separated by block barriers).  The per-point
arithmetic and the buffers are those of the launch-per-pass path, so the
results must be the same bits: both precision classes, both methods, every
boundary code (BC 4 included), odd and even step counts (the mixed state
pair flips per step), and sizes up to the limit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(n, method, prec, BC, steps, small_max):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    x = np.linspace(-20.0, 20.0, n)
    U = np.tanh(x / 1.4) * np.exp(0.3j * x) + 0.05
    V = 0.002 * x * x
    old = autotune.get_knob("small1d.max_points")
    try:
        autotune.set_knob("small1d.max_points", small_max)
        with ng.Solver((n,), method=method, precision=prec, BC=BC, s=-1.0, a=1.0,
                       h2=(x[1] - x[0]) ** 2, k=0.2 * (x[1] - x[0]) ** 2) as sv:
            sv.upload(U, V)
            sv.run(steps)
            sv.run(3)
            return np.ascontiguousarray(sv.download())
    finally:
        autotune.set_knob("small1d.max_points", old)


@pytest.mark.parametrize("prec", [1, 3])
@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("BC", [1, 2, 3, 4])
@pytest.mark.parametrize("n,steps", [(64, 7), (1024, 20), (4096, 9)])
def test_small1d_matches_stage_launches(gpu_lib, n, steps, BC, method, prec):
    ref = _run(n, method, prec, BC, steps, 0)
    got = _run(n, method, prec, BC, steps, 4096)
    assert np.all(np.isfinite(ref))
    assert np.array_equal(got.view(np.float64), ref.view(np.float64)), \
        "max |diff| %g" % np.max(np.abs(got - ref))


def test_small1d_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("small1d.max_points", 1 << 20)
