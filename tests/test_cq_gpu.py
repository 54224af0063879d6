"""2D cubic-quintic 2SHOC (src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c) on the
GPU: bit-identical to the C oracle (itself pinned to the reference file), also
through the MEX gateway."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
dp = ctypes.POINTER(ctypes.c_double)


def bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.float64),
                          np.ascontiguousarray(b).view(np.float64))


@pytest.mark.parametrize("shape", [(3, 3), (9, 7), (33, 17), (128, 96)])
@pytest.mark.parametrize("BC", [1, 2, 3])
@pytest.mark.parametrize("s2", [0.0, 0.4, -0.7])
def test_cq2d_gpu_matches_oracle(gpu_lib, shape, BC, s2):
    import nlsemagic_gb300 as ng
    rng = np.random.default_rng(shape[0] + BC)
    U = (1 + 0.3 * rng.standard_normal(shape)) + 0.3j * rng.standard_normal(shape)
    V = 0.1 * rng.random(shape)
    args = (U, V, -1.0, s2, 1.2, 0.09, BC, 9, 0.003)
    got = ng.CQNLSE2D_TAKE_STEPS_2SHOC(*args)
    want = oracle.cq2d(*args, flags=oracle.MSD_GUARD)
    assert bits_equal(got, want)


def test_cq2d_zero_neighbour_guard(gpu_lib):
    import nlsemagic_gb300 as ng
    U = np.ones((8, 9), complex)
    U[1, 1] = 0.0  # MSD neighbour of the corner (0, 0)
    V = np.zeros(U.shape)
    got = ng.CQNLSE2D_TAKE_STEPS_2SHOC(U, V, -1.0, 0.2, 1.0, 0.04, 2, 3, 0.001)
    assert np.all(np.isfinite(got))
    assert bits_equal(got, oracle.cq2d(U, V, -1.0, 0.2, 1.0, 0.04, 2, 3, 0.001, flags=1))


def test_cq2d_mex_gateway(gpu_lib, tmp_path):
    import nlsemagic_gb300 as ng
    libdir = os.path.join(ROOT, "nlsemagic_gb300")
    so = str(tmp_path / "cq.so")
    cmd = ["gcc", "-std=gnu89", "-O2", "-fPIC", "-shared", "-I",
           os.path.join(ROOT, "oracle", "mexshim"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "nlsemagic_gb300", "mex", "CQNLSE2D_TAKE_STEPS_2SHOC_CUDA_D.c"),
           os.path.join(ROOT, "oracle", "mexshim", "mexshim.c"), "-L", libdir, "-lnlse_gb300",
           "-Wl,-rpath," + libdir, "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so, mode=ctypes.RTLD_LOCAL)
    f = lib.mex_call_cq2d
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_longlong), dp, dp, dp] + [ctypes.c_double] * 4 + \
        [ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, dp]
    rng = np.random.default_rng(2)
    shape = (21, 13)
    U = (1 + 0.2 * rng.standard_normal(shape)) + 0.2j * rng.standard_normal(shape)
    V = 0.1 * rng.random(shape)
    re = np.ascontiguousarray(U.real.ravel(order="F"))
    im = np.ascontiguousarray(U.imag.ravel(order="F"))
    vv = np.ascontiguousarray(V.ravel(order="F"))
    outr, outi = np.empty(U.size), np.empty(U.size)
    cd = (ctypes.c_longlong * 2)(*shape)
    rc = f(cd, re.ctypes.data_as(dp), im.ctypes.data_as(dp), vv.ctypes.data_as(dp), -1.0, 0.5,
           1.1, 0.0625, 2, 6, 0.002, outr.ctypes.data_as(dp), outi.ctypes.data_as(dp))
    assert rc == 0
    got = (outr + 1j * outi).reshape(shape, order="F")
    assert bits_equal(got, ng.CQNLSE2D_TAKE_STEPS_2SHOC(U, V, -1.0, 0.5, 1.1, 0.0625, 2, 6, 0.002))
