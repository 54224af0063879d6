"""Mixed-precision 3D 2SHOC: the fused interior kernel (face ghosts and face
updates inside it, one launch per RK4 stage) gives the same bits as the
three-kernel form (face ghosts, interior, faces) for every boundary
condition, on grids that exercise the tile shifts: M-1 a multiple of 32
(x tiles start two cells early; odd M also takes the plain-load staging),
N-1 a multiple of the tile height (y tiles start one row early), L-1 a
multiple of the z chunk (the last chunk absorbs the z = L-1 face), and the
thinnest grids (3 cells)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [  # (L, N, M) as the solver takes them; zc = z-chunk override (0: heuristic)
    ((19, 17, 20), 0),
    ((21, 12, 33), 0),
    ((10, 9, 34), 0),
    ((37, 40, 64), 0),
    ((3, 3, 3), 0),
    ((6, 4, 5), 0),
    ((49, 25, 66), 16),
    ((33, 41, 65), 8),
]


def _run(shape, BC, fuse, zc, steps=3):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    # a smooth field: the MSD boundary amplifies grid-scale noise, so random
    # data would overflow within a few steps on either form
    z, y, x = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    U = (0.8 + 0.2 * np.cos(2.1 * x + 0.3) * np.cos(1.7 * y) * np.cos(1.3 * z + 0.5)
         + 0.15j * np.sin(1.9 * x + 1.1 * y + 0.7 * z))
    V = 0.5 + 0.5 * (x - 0.5) ** 2 + 0.3 * (y - 0.4) ** 2 + 0.2 * z
    old = {k: autotune.get_knob(k) for k in ("wide.fuse", "wide.zc")}
    try:
        autotune.set_knob("wide.fuse", fuse)
        autotune.set_knob("wide.zc", zc)
        with ng.Solver(shape, method=2, precision=ng.PREC_MIXED, BC=BC, s=-1.0, a=1.0,
                       h2=0.09, k=0.004) as sv:
            lps = sv.launches_per_step
            sv.upload(U, V)
            sv.run(steps)
            out = np.ascontiguousarray(sv.download())
    finally:
        for k, v in old.items():
            autotune.set_knob(k, v)
    return out, lps


@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("shape,zc", SHAPES)
def test_fused_matches_three_kernel_form(gpu_lib, shape, zc, BC):
    fused, lf = _run(shape, BC, 1, zc)
    split, ls = _run(shape, BC, 0, zc)
    assert lf == 4 and ls == 12
    assert np.all(np.isfinite(fused))
    assert np.array_equal(fused.view(np.float64), split.view(np.float64)), \
        "max |diff| %g" % np.max(np.abs(fused - split))


def test_fuse_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("wide.fuse", 2)
