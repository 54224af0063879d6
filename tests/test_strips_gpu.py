"""Mixed-precision 3D 2SHOC with x-face strips: the x faces' own lo, K and
V kept in face-indexed arrays, which the face kernel reads and writes in
place of the full arrays' strided x faces (K there lives in the strip
only).

The same values, so the results must be bit-identical to the run without
strips: every boundary condition, grids with and without interior tiles,
graphs, runs split into calls, a new state uploaded into a running solver,
and the knob switched off and on between runs (the strips are refilled)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(20, 17, 19), (34, 12, 33), (40, 40, 40), (3, 4, 5), (64, 33, 70), (96, 64, 130),
          (66, 20, 21), (21, 12, 33)]


def _case(shape, phase=0.0):
    z, y, x = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    U = (0.8 + 0.2 * np.cos(2.1 * x + 0.3 + phase) * np.cos(1.7 * y) * np.cos(1.3 * z + 0.5)
         + 0.15j * np.sin(1.9 * x + 1.1 * y + 0.7 * z))
    V = 0.5 + 0.5 * (x - 0.5) ** 2 + 0.3 * (y - 0.4) ** 2 + 0.2 * z
    return U, V


def _solver(ng, shape, BC):
    return ng.Solver(shape, method=2, precision=ng.PREC_MIXED, BC=BC, s=-1.0, a=1.0, h2=0.09,
                     k=0.004)


def _run(shape, BC, strips, calls=(3,), graph_steps=0):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    U, V = _case(shape)
    old = autotune.get_knob("wide.strips")
    try:
        autotune.set_knob("wide.strips", strips)
        with _solver(ng, shape, BC) as sv:
            if graph_steps:
                sv.set_graph_steps(graph_steps)
            sv.upload(U, V)
            for n in calls:
                sv.run(n)
            return np.ascontiguousarray(sv.download())
    finally:
        autotune.set_knob("wide.strips", old)


def _same(a, b):
    return np.array_equal(a.view(np.float64), b.view(np.float64))


@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("shape", SHAPES)
def test_strips_match_full_arrays(gpu_lib, shape, BC):
    ref = _run(shape, BC, 0)
    assert np.all(np.isfinite(ref))
    got = _run(shape, BC, 1)
    assert _same(got, ref), "max |diff| %g" % np.max(np.abs(got - ref))


@pytest.mark.parametrize("BC", [2, 3])
@pytest.mark.parametrize("shape", [(40, 40, 40), (96, 64, 130)])
def test_strips_graphs_and_split_runs(gpu_lib, shape, BC):
    ref = _run(shape, BC, 0, calls=(7,))
    for graph_steps, calls in ((2, (7,)), (3, (7,)), (0, (1, 2, 4)), (2, (3, 4))):
        got = _run(shape, BC, 1, calls=calls, graph_steps=graph_steps)
        assert _same(got, ref), (graph_steps, calls)


def test_strips_refilled_after_upload_and_knob_changes(gpu_lib):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    shape, BC = (64, 33, 70), 2
    U1, V = _case(shape)
    U2, _ = _case(shape, phase=0.7)
    old = autotune.get_knob("wide.strips")

    def seq(knobs):
        with _solver(ng, shape, BC) as sv:
            sv.upload(U1, V)
            autotune.set_knob("wide.strips", knobs[0])
            sv.run(2)
            autotune.set_knob("wide.strips", knobs[1])
            sv.run(3)  # strips refilled if they were off
            sv.upload(U2, V)  # a new state: refilled before the next stage
            autotune.set_knob("wide.strips", knobs[2])
            sv.run(2)
            return np.ascontiguousarray(sv.download())

    try:
        ref = seq((0, 0, 0))
        for knobs in ((1, 1, 1), (1, 0, 1), (0, 1, 1), (1, 1, 0)):
            assert _same(seq(knobs), ref), knobs
    finally:
        autotune.set_knob("wide.strips", old)


def test_strips_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("wide.strips", 2)
