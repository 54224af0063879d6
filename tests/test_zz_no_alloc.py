"""The allocation-free entry point, nlse_take_steps_noalloc.

For callers that cannot allocate device memory: plug-ins whose host
application owns every device allocation (a MEX function on MATLAB gpuArray
data, a framework with its own memory pool) and real-time loops that may not
allocate after start-up.  They pass their own device buffers and the library
keeps its RK4 scratch in a fixed device array.

Checked here through the C ABI, on two calls in a row with different inputs
(the shared scratch keeps the previous call's contents, which must not leak
into the next result):
* against the ordinary entry point, nlse_take_steps, bit for bit (FP64), on
  small grids and on grids at the 2^18-point limit, where nlse_take_steps
  runs other kernels (the tiled 3D and 2D forms) than the allocation-free
  path;
* against the C oracle directly, bit for bit;
* a repeated call changes the device's free memory by nothing.
This file is collected last, and works alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

S, A, H2, K = -1.0, 1.1, 0.09, 0.002


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    U = (1 + 0.2 * rng.standard_normal(shape)) + 0.2j * rng.standard_normal(shape)
    V = 0.1 * rng.random(shape)
    return U, V


class _DeviceCall:
    """Device buffers for one grid, made before the call so that timing or
    memory checks around the call see only the library's work."""

    def __init__(self, U, V):
        import torch
        from nlsemagic_gb300.api import planar
        re, im = planar(U)
        self.shape = U.shape
        self.d = [torch.from_numpy(x).cuda()
                  for x in (re, im, np.ascontiguousarray(V.ravel(order="F")))]
        self.outr = torch.empty_like(self.d[0])
        self.outi = torch.empty_like(self.d[0])
        torch.cuda.synchronize()

    def run(self, lib, prob, chunk):
        import torch
        st = torch.cuda.current_stream()
        rc = lib.nlse_take_steps_noalloc(ctypes.byref(prob), self.d[0].data_ptr(),
                                         self.d[1].data_ptr(), self.d[2].data_ptr(),
                                         self.outr.data_ptr(), self.outi.data_ptr(), chunk,
                                         st.cuda_stream)
        assert rc == 0, lib.nlse_last_error_string()
        st.synchronize()

    def result(self):
        return (self.outr.cpu().numpy() + 1j * self.outi.cpu().numpy()).reshape(
            self.shape, order="F")


@pytest.mark.parametrize("shape,method,BC", [
    ((300,), 2, 2), ((40, 37), 1, 3), ((12, 9, 10), 2, 2), ((64,), 1, 4),
    ((512, 512), 2, 1), ((64, 64, 64), 2, 2), ((1 << 18,), 1, 2)])
def test_noalloc_matches_take_steps_two_calls(gpu_lib, shape, method, BC):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.api import grid_dims, make_problem
    lib = ng.load()
    ndim, dims = grid_dims(shape)
    for call, seed in enumerate((1, 2)):
        U, V = _case(shape, 100 * seed + len(shape))
        chunk = 6 + call
        prob = make_problem(ndim, dims, method, ng.PREC_DOUBLE, BC, S, A, H2, K)
        dc = _DeviceCall(U, V)
        dc.run(lib, prob, chunk)
        got = dc.result()
        want = ng.take_steps(U, V, S, A, H2, BC, chunk, K, method=method,
                             precision=ng.PREC_DOUBLE)
        assert bits_equal(got, want), "call %d differs from nlse_take_steps" % call
        ref = oracle.take_steps(U, V, S, A, H2, BC, chunk, K, method=method, precision=2,
                                flags=oracle.MSD_GUARD)
        assert bits_equal(got, ref), "call %d differs from the oracle" % call


def test_noalloc_repeat_call_allocates_nothing(gpu_lib):
    import torch

    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.api import grid_dims, make_problem
    lib = ng.load()
    shape = (48, 40, 36)
    ndim, dims = grid_dims(shape)
    U, V = _case(shape, 7)
    prob = make_problem(ndim, dims, 2, ng.PREC_DOUBLE, 2, S, A, H2, K)
    dc = _DeviceCall(U, V)
    dc.run(lib, prob, 3)  # first call: kernels load, scratch address looked up
    first = dc.result()
    free0 = torch.cuda.mem_get_info()[0]
    dc.run(lib, prob, 3)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, "device free memory changed by %d bytes" % (free0 - free1)
    assert bits_equal(dc.result(), first)


def test_noalloc_rejects_oversize_grid(gpu_lib):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300.api import make_problem
    lib = ng.load()
    n = (1 << 18) + 1
    prob = make_problem(1, (n, 1, 1), 1, ng.PREC_DOUBLE, 1, -1.0, 1.0, 0.01, 1e-3)
    rc = lib.nlse_take_steps_noalloc(ctypes.byref(prob), 8, 8, 8, 8, 8, 1, None)
    assert rc == ng._lib.NLSE_ERR_CAPACITY
    assert b"NLSE_NOALLOC_MAX_POINTS" in lib.nlse_last_error_string()
