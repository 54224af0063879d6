"""nlse_device_fp64_rates: the FP64 FMA and add rates of the current device,
measured by a timed kernel (the compute bound the exact FP64 class is
compared with).  The rates are positive and finite, an FMA issues at least
as fast as an add would on any FP64 pipe (it is one instruction doing two
flops), and two calls agree within the noise of a timed kernel."""
import ctypes
import math

import pytest

pytestmark = pytest.mark.gpu


def _rates(lib):
    fma, add = ctypes.c_double(), ctypes.c_double()
    rc = lib.nlse_device_fp64_rates(ctypes.byref(fma), ctypes.byref(add))
    assert rc == 0, lib.nlse_last_error_string()
    return fma.value, add.value


def test_fp64_rates_are_measured(gpu_lib):
    fma1, add1 = _rates(gpu_lib)
    fma2, add2 = _rates(gpu_lib)
    for v in (fma1, add1, fma2, add2):
        assert math.isfinite(v) and v > 1e9  # well above a gigaop per second
    assert fma1 >= 0.5 * add1
    assert abs(fma1 - fma2) <= 0.2 * max(fma1, fma2)
    assert abs(add1 - add2) <= 0.2 * max(add1, add2)


def test_fp64_rates_reject_null(gpu_lib):
    out = ctypes.c_double()
    rc = gpu_lib.nlse_device_fp64_rates(None, ctypes.byref(out))
    assert rc != 0
