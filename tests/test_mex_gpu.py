"""MATLAB-facing boundary: the MEX gateway sources in nlsemagic_gb300/mex,
compiled against the oracle's mex.h stand-in (MATLAB is not available) and
called through it with the reference MEX argument lists, must give exactly
the results of the library's own entry point."""
import ctypes
import glob
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MEXDIR = os.path.join(ROOT, "nlsemagic_gb300", "mex")
dp = ctypes.POINTER(ctypes.c_double)


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


@pytest.fixture(scope="module")
def gateways(tmp_path_factory, gpu_lib):
    out = tmp_path_factory.mktemp("mex")
    libdir = os.path.join(ROOT, "nlsemagic_gb300")
    built = {}
    for src in sorted(glob.glob(os.path.join(MEXDIR, "*.c"))):
        name = os.path.basename(src)[:-2]
        so = str(out / (name + ".so"))
        cmd = ["gcc", "-std=gnu89", "-O2", "-fPIC", "-shared", "-I", os.path.join(ROOT, "oracle", "mexshim"),
               "-I", os.path.join(ROOT, "include"), src,
               os.path.join(ROOT, "oracle", "mexshim", "mexshim.c"), "-L", libdir, "-lnlse_gb300",
               "-Wl,-rpath," + libdir, "-o", so]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        lib = ctypes.CDLL(so, mode=ctypes.RTLD_LOCAL)
        f = lib.mex_call_take_steps
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), dp, dp, dp, ctypes.c_double,
                      ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                      ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
        built[name] = lib
    return built


def call(lib, U, V, args, precision=0, method=0, nrhs=8):
    from nlsemagic_gb300.api import planar
    re, im = planar(U)
    vv = np.ascontiguousarray(V.ravel(order="F"))
    dims = U.shape if U.ndim > 1 else (U.shape[0],)
    cd = (ctypes.c_longlong * len(dims))(*dims)
    outr = np.empty_like(re)
    outi = np.empty_like(im)
    s, a, h2, BC, chunk, k = args
    rc = lib.mex_call_take_steps(len(dims), cd, re.ctypes.data_as(dp), im.ctypes.data_as(dp),
                                 vv.ctypes.data_as(dp), s, a, h2, BC, chunk, k, precision, method,
                                 nrhs, outr.ctypes.data_as(dp), outi.ctypes.data_as(dp))
    return rc, (outr + 1j * outi).reshape(U.shape, order="F")


SHAPES = {1: (41,), 2: (13, 17), 3: (9, 8, 7)}


def test_every_v1_gateway_matches_library(gateways):
    import nlsemagic_gb300 as ng
    rng = np.random.default_rng(3)
    names = [n for n in gateways if n.startswith("NLSE") and "_CUDA_" in n]
    assert len(names) == 18
    for name in names:
        ndim = int(name[4])
        method = 2 if "2SHOC" in name else 1
        prec = {"D": 2, "F": 1, "M": 3}[name[-1]]
        shape = SHAPES[ndim]
        U = (1 + 0.2 * rng.standard_normal(shape)) + 0.2j * rng.standard_normal(shape)
        V = 0.1 * rng.random(shape)
        args = (-1.0, 1.2, 0.1, 2, 5, 0.002)
        rc, got = call(gateways[name], U, V, args)
        assert rc == 0, name
        want = ng.take_steps(U, V, *args[:4], args[4], args[5], method=method, precision=prec)
        assert bits_equal(got, want), name


def test_v2_gateways_and_error_path(gateways):
    import nlsemagic_gb300 as ng
    rng = np.random.default_rng(4)
    for ndim in (1, 2, 3):
        lib = gateways["NLSEmagic%dD_Take_Steps_GPU" % ndim]
        shape = SHAPES[ndim]
        U = (1 + 0.2 * rng.standard_normal(shape)) + 0.2j * rng.standard_normal(shape)
        V = 0.1 * rng.random(shape)
        args = (1.0, 0.8, 0.1, 1, 4, 0.002)
        for prec in (1, 2, 3):
            for method in (1, 2):
                rc, got = call(lib, U, V, args, precision=prec, method=method, nrhs=10)
                assert rc == 0
                want = ng.take_steps(U, V, *args[:4], args[4], args[5], method=method,
                                     precision=prec)
                assert bits_equal(got, want)
        # an invalid boundary code surfaces as a MATLAB error, not a crash
        rc, _ = call(lib, U, V, (1.0, 0.8, 0.1, 9, 4, 0.002), precision=2, method=1, nrhs=10)
        assert rc == -3
