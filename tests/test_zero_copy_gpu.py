"""Page-locked host arrays: upload and download read and write them in place
(the layout-conversion kernels access the mapped host memory), pageable
arrays go through the device staging buffer.  Both give the same bits, in
every precision class and dimension, with the zero-copy knob on or off;
real input (no imaginary array) too."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [((300,), 2, 2), ((40, 33), 2, 1), ((12, 10, 9), 2, 2), ((45, 38), 1, 3), ((500,), 1, 1)]


def _pinned(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).pin_memory()


def _ptr(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))


def _field(shape):
    rng = np.random.default_rng(sum(shape))
    U = (0.9 + 0.1 * rng.standard_normal(shape)) + 0.1j * rng.standard_normal(shape)
    V = 0.05 * rng.random(shape)
    return U, V


@pytest.mark.parametrize("prec", [2, 3, 1])
@pytest.mark.parametrize("shape,method,BC", CASES)
def test_pinned_and_pageable_same_bits(gpu_lib, shape, method, BC, prec):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import autotune
    from nlsemagic_gb300.api import planar
    U, V = _field(shape)
    kw = dict(method=method, precision=prec, BC=BC, s=-1.0, a=1.0, h2=0.09, k=0.002)
    with ng.Solver(shape, **kw) as sv:  # pageable: staged copies
        sv.upload(U, V)
        sv.run(5)
        want = sv.download()
    re, im = planar(U)
    vv = np.asarray(V, dtype=np.float64).ravel(order="F")
    for zc in (1, 0):
        old = autotune.get_knob("io.zero_copy")
        try:
            autotune.set_knob("io.zero_copy", zc)
            hre, him, hv = _pinned(re), _pinned(im), _pinned(vv)
            ore, oim = _pinned(np.zeros(re.size)), _pinned(np.zeros(re.size))
            with ng.Solver(shape, **kw) as sv:
                ng._lib.check(sv._lib.nlse_solver_upload(sv._h, _ptr(hre), _ptr(him), _ptr(hv)))
                sv.run(5)
                ng._lib.check(sv._lib.nlse_solver_download(sv._h, _ptr(ore), _ptr(oim)))
            got = (ore.numpy() + 1j * oim.numpy()).reshape(shape, order="F")
        finally:
            autotune.set_knob("io.zero_copy", old)
        assert np.array_equal(np.ascontiguousarray(got).view(np.float64),
                              np.ascontiguousarray(want).view(np.float64))


def test_pinned_real_input(gpu_lib):
    # a real U (no imaginary array): the imaginary part starts at zero
    import nlsemagic_gb300 as ng
    U, V = _field((64, 40))
    kw = dict(method=2, precision=3, BC=2, s=-1.0, a=1.0, h2=0.09, k=0.002)
    with ng.Solver(U.shape, **kw) as sv:
        sv.upload(U.real, V)
        sv.run(3)
        want = sv.download()
    hre = _pinned(U.real.ravel(order="F"))
    hv = _pinned(V.ravel(order="F"))
    with ng.Solver(U.shape, **kw) as sv:
        ng._lib.check(sv._lib.nlse_solver_upload(sv._h, _ptr(hre), None, _ptr(hv)))
        sv.run(3)
        got = sv.download()
    assert np.array_equal(np.ascontiguousarray(got).view(np.float64),
                          np.ascontiguousarray(want).view(np.float64))


def test_zero_copy_knob_range(gpu_lib):
    from nlsemagic_gb300 import autotune
    with pytest.raises(Exception):
        autotune.set_knob("io.zero_copy", 2)
