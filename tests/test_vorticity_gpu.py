"""3D vorticity (post-chunk analysis, src/NLSEmagic3D/rmc_vorticity3D.c):
the GPU kernels against the C oracle, bit for bit at every point; the MEX
gateway and the resident-solver entry point against the library call."""
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
    return np.array_equal(np.asarray(a).view(np.int64), np.asarray(b).view(np.int64))


@pytest.mark.parametrize("shape", [(3, 3, 3), (5, 6, 7), (33, 17, 9), (64, 40, 21),
                                   (4, 70, 5)])
@pytest.mark.parametrize("real", [False, True])
def test_vorticity_gpu_matches_oracle(gpu_lib, shape, real):
    import nlsemagic_gb300 as ng
    rng = np.random.default_rng(sum(shape) + real)
    U = rng.standard_normal(shape) + (0 if real else 1j * rng.standard_normal(shape))
    U.flat[7] = 0.0
    lh2, veps = 1.0 / (2 * 0.27), 1e-7
    got = ng.rmc_vorticity3D(U, lh2, veps)
    want = oracle.vorticity3d(U, lh2, veps)
    for g, w in zip(got, want):
        assert bits_equal(g, w)


def test_vorticity_rejects_bad_arguments(gpu_lib):
    import nlsemagic_gb300 as ng
    with pytest.raises(ValueError):
        ng.rmc_vorticity3D(np.ones((4, 4)), 1.0, 1e-6)
    with pytest.raises(ng.NLSEError):
        ng.rmc_vorticity3D(np.ones((2, 4, 4), complex), 1.0, 1e-6)


def test_solver_vorticity_equals_download_then_vorticity(gpu_lib):
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import workloads as W
    w = W.vortex_rings_3d(n=40, steps=6)
    for prec in (ng.PREC_DOUBLE, ng.PREC_MIXED):
        with ng.Solver(w.U.shape, method=2, precision=prec, BC=w.BC, s=w.s, a=w.a, h2=w.h2,
                       k=w.k) as s:
            s.upload(w.U, w.V)
            s.run(w.steps)
            got = s.vorticity(1e-9)
            want = ng.rmc_vorticity3D(s.download(), 1.0 / (2.0 * np.sqrt(w.h2)), 1e-9)
        for g, x in zip(got, want):
            assert bits_equal(g, x)


def test_vorticity_mex_gateway(gpu_lib, tmp_path):
    import nlsemagic_gb300 as ng
    libdir = os.path.join(ROOT, "nlsemagic_gb300")
    so = str(tmp_path / "rmc_vorticity3D.so")
    cmd = ["gcc", "-std=gnu89", "-O2", "-fPIC", "-shared", "-I",
           os.path.join(ROOT, "oracle", "mexshim"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "nlsemagic_gb300", "mex", "rmc_vorticity3D.c"),
           os.path.join(ROOT, "oracle", "mexshim", "mexshim.c"), "-L", libdir, "-lnlse_gb300",
           "-Wl,-rpath," + libdir, "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(so, mode=ctypes.RTLD_LOCAL)
    f = lib.mex_call_vorticity
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_longlong), dp, dp, ctypes.c_double, ctypes.c_double,
                  dp, dp, dp, dp]
    rng = np.random.default_rng(5)
    shape = (11, 9, 7)
    U = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    re = np.ascontiguousarray(U.real.ravel(order="F"))
    im = np.ascontiguousarray(U.imag.ravel(order="F"))
    outs = [np.empty(U.size) for _ in range(4)]
    cd = (ctypes.c_longlong * 3)(*shape)
    rc = f(cd, re.ctypes.data_as(dp), im.ctypes.data_as(dp), 1.7, 1e-8,
           *(o.ctypes.data_as(dp) for o in outs))
    assert rc == 0
    want = ng.rmc_vorticity3D(U, 1.7, 1e-8)
    for o, w in zip(outs, want):
        assert bits_equal(o.reshape(shape, order="F"), w)
