"""The allocation-free entry point, nlse_take_steps_noalloc.

For callers that cannot allocate device memory (work captured into a CUDA
graph, plug-ins whose host owns every device allocation, real-time loops):
they pass their own device buffers and the library keeps its RK4 scratch in
a fixed device array.  Checked here through the C ABI against the ordinary
entry point, nlse_take_steps, on two calls in a row with different inputs
(the shared scratch keeps the previous call's contents, which must not leak
into the next result).  FP64 results must be bit-identical.  This file is
collected last, and works alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    U = (1 + 0.2 * rng.standard_normal(shape)) + 0.2j * rng.standard_normal(shape)
    V = 0.1 * rng.random(shape)
    return U, V


def _noalloc(lib, prob, U, V, chunk):
    import torch
    from nlsemagic_gb300.api import planar
    re, im = planar(U)
    d = [torch.from_numpy(x).cuda() for x in (re, im, np.ascontiguousarray(V.ravel(order="F")))]
    outr = torch.empty_like(d[0])
    outi = torch.empty_like(d[0])
    st = torch.cuda.current_stream()
    rc = lib.nlse_take_steps_noalloc(ctypes.byref(prob), d[0].data_ptr(), d[1].data_ptr(),
                                     d[2].data_ptr(), outr.data_ptr(), outi.data_ptr(), chunk,
                                     st.cuda_stream)
    assert rc == 0, lib.nlse_last_error_string()
    st.synchronize()
    return (outr.cpu().numpy() + 1j * outi.cpu().numpy()).reshape(U.shape, order="F")


@pytest.mark.parametrize("shape,method,BC", [((300,), 2, 2), ((40, 37), 1, 3), ((12, 9, 10), 2, 2),
                                             ((64,), 1, 4)])
def test_noalloc_matches_take_steps_two_calls(gpu_lib, shape, method, BC):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.api import grid_dims, make_problem
    lib = ng.load()
    ndim, dims = grid_dims(shape)
    for call, seed in enumerate((1, 2)):
        U, V = _case(shape, 100 * seed + len(shape))
        prob = make_problem(ndim, dims, method, ng.PREC_DOUBLE, BC, -1.0, 1.1, 0.09, 0.002)
        got = _noalloc(lib, prob, U, V, 6 + call)
        want = ng.take_steps(U, V, -1.0, 1.1, 0.09, BC, 6 + call, 0.002, method=method,
                             precision=ng.PREC_DOUBLE)
        assert bits_equal(got, want), "call %d" % call


def test_noalloc_rejects_oversize_grid(gpu_lib):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.api import make_problem
    lib = ng.load()
    n = (1 << 18) + 1
    prob = make_problem(1, (n, 1, 1), 1, ng.PREC_DOUBLE, 1, -1.0, 1.0, 0.01, 1e-3)
    rc = lib.nlse_take_steps_noalloc(ctypes.byref(prob), 8, 8, 8, 8, 8, 1, None)
    assert rc == ng._lib.NLSE_ERR_CAPACITY
    assert b"NLSE_NOALLOC_MAX_POINTS" in lib.nlse_last_error_string()
