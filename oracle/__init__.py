"""CPU oracle for the NLSEmagic RK4 chunk integrators.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package; the product library
(``nlsemagic_gb300``) never does and has no CPU fallback.

* :func:`take_steps` -- this project's C restatement (``nlse_oracle.c``),
  available on every machine after :func:`oracle.build.build_port`.
* :func:`ref_take_steps` -- the reference's own unmodified C integrators,
  built against ``mexshim`` into ``oracle/_ref`` where the reference checkout
  exists (see ``oracle/build.py``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

MSD_GUARD = 1
REF_QUIRKS = 2

_dp = ctypes.POINTER(ctypes.c_double)
_port = None
_refs = {}


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _load_port():
    global _port
    if _port is None:
        path = _build.build_port()
        lib = ctypes.CDLL(path)
        f = lib.nlse_oracle_take_steps
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                      _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                      ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp, ctypes.c_int]
        _port = lib
    return _port


def set_threads(n):
    """OpenMP threads that one take_steps call spreads its grid sweeps over
    (default 1, serial like the reference).  The result bits do not depend
    on it: every sweep writes each point from values no other point of the
    same sweep writes."""
    f = _load_port().nlse_oracle_set_threads
    f.restype = None
    f.argtypes = [ctypes.c_int]
    f(int(n))


def _dims_of(U):
    """MATLAB dims of a MATLAB-shaped array: shape (M,), (M, N) or (M, N, L),
    first index fastest (Fortran order)."""
    return tuple(int(d) for d in U.shape)


def _planes(U, V):
    U = np.asarray(U)
    Ur = np.ascontiguousarray(np.real(U).ravel(order="F"), dtype=np.float64)
    Ui = np.ascontiguousarray(np.imag(U).ravel(order="F") if np.iscomplexobj(U)
                              else np.zeros(U.size), dtype=np.float64)
    Vv = np.ascontiguousarray(np.asarray(V, dtype=np.float64).ravel(order="F"))
    return Ur, Ui, Vv


def take_steps(U, V, s, a, h2, BC, chunk, k, method=1, precision=2, flags=MSD_GUARD):
    """Run the C restatement.  U complex (or real), V real, MATLAB-shaped
    numpy arrays: (M,), (M, N) or (M, N, L), first index fastest.  Returns a
    new complex128 array of U's shape."""
    U = np.asarray(U)
    Ur, Ui, Vv = _planes(U, V)
    dims = _dims_of(U)
    cd = (ctypes.c_longlong * len(dims))(*dims)
    outr = np.empty_like(Ur)
    outi = np.empty_like(Ui)
    rc = _load_port().nlse_oracle_take_steps(len(dims), int(method), int(precision), cd,
                                             _ptr(Ur), _ptr(Ui), _ptr(Vv), float(s), float(a),
                                             float(h2), int(BC), int(chunk), float(k),
                                             _ptr(outr), _ptr(outi), int(flags))
    if rc != 0:
        raise ValueError("oracle rejected arguments (code %d)" % rc)
    return (outr + 1j * outi).reshape(U.shape, order="F")


def ref_name(ndim, method, precision):
    return "NLSE%dD_TAKE_STEPS_%s%s" % (ndim, "CD" if method == 1 else "2SHOC",
                                        "_F" if precision == 1 else "")


def ref_available():
    return _build.reference_available()


def _load_ref(name):
    if name not in _refs:
        libs = _build.build_ref()
        if name not in libs:
            raise RuntimeError("reference integrator %s is not available here" % name)
        lib = ctypes.CDLL(libs[name], mode=ctypes.RTLD_LOCAL)
        f = lib.ref_take_steps
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), _dp, _dp, _dp,
                      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                      ctypes.c_int, ctypes.c_double, _dp, _dp]
        _refs[name] = lib
    return _refs[name]


def ref_take_steps(U, V, s, a, h2, BC, chunk, k, method=1, precision=2):
    """Run the reference's own C integrator (unmodified, via the mex shim)."""
    U = np.asarray(U)
    Ur, Ui, Vv = _planes(U, V)
    dims = _dims_of(U)
    cd = (ctypes.c_longlong * len(dims))(*dims)
    outr = np.empty_like(Ur)
    outi = np.empty_like(Ui)
    lib = _load_ref(ref_name(len(dims), method, precision))
    rc = lib.ref_take_steps(len(dims), cd, _ptr(Ur), _ptr(Ui), _ptr(Vv), float(s), float(a),
                            float(h2), int(BC), int(chunk), float(k), _ptr(outr), _ptr(outi))
    if rc != 0:
        raise RuntimeError("reference call failed (code %d)" % rc)
    return (outr + 1j * outi).reshape(U.shape, order="F")


def vorticity3d(U, lh2, veps):
    """C restatement of the 3D vorticity routine: U MATLAB-shaped (M, N, L),
    lh2 = 1/(2h).  Returns (wx, wy, wz, W), each real of U's shape."""
    U = np.asarray(U)
    if U.ndim != 3:
        raise ValueError("vorticity3d needs a 3D array")
    M, N, L = (int(d) for d in U.shape)
    Ur, Ui, _ = _planes(U, np.zeros(U.shape))
    lib = _load_port()
    f = lib.nlse_oracle_vorticity3d
    f.restype = None
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                  ctypes.c_double, _dp, _dp, _dp, _dp]
    outs = [np.empty(U.size) for _ in range(4)]
    f(M, N, L, _ptr(Ur), _ptr(Ui), float(lh2), float(veps), *(_ptr(o) for o in outs))
    return tuple(o.reshape(U.shape, order="F") for o in outs)


def ref_vorticity3d(U, lh2, veps):
    """The reference's own rmc_vorticity3D MEX function (via the shim)."""
    U = np.asarray(U)
    if "rmc_vorticity3D" not in _refs:
        libs = _build.build_ref()
        if "rmc_vorticity3D" not in libs:
            raise RuntimeError("reference vorticity routine is not available here")
        lib = ctypes.CDLL(libs["rmc_vorticity3D"], mode=ctypes.RTLD_LOCAL)
        f = lib.mex_call_vorticity
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(ctypes.c_longlong), _dp, _dp, ctypes.c_double,
                      ctypes.c_double, _dp, _dp, _dp, _dp]
        _refs["rmc_vorticity3D"] = lib
    lib = _refs["rmc_vorticity3D"]
    Ur, Ui, _ = _planes(U, np.zeros(U.shape))
    cd = (ctypes.c_longlong * 3)(*(int(d) for d in U.shape))
    outs = [np.empty(U.size) for _ in range(4)]
    rc = lib.mex_call_vorticity(cd, _ptr(Ur), _ptr(Ui) if np.iscomplexobj(U) else None,
                                float(lh2), float(veps), *(_ptr(o) for o in outs))
    if rc != 0:
        raise RuntimeError("reference vorticity call failed (code %d)" % rc)
    return tuple(o.reshape(U.shape, order="F") for o in outs)


def cq2d(U, V, s1, s2, a, h2, BC, chunk, k, flags=MSD_GUARD):
    """C restatement of the 2D cubic-quintic 2SHOC integrator (FP64).  U
    MATLAB-shaped (M, N)."""
    U = np.asarray(U)
    M, N = (int(d) for d in U.shape)
    Ur, Ui, Vv = _planes(U, V)
    lib = _load_port()
    f = lib.nlse_oracle_cq2d
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp] + [ctypes.c_double] * 4 + \
        [ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp, ctypes.c_int]
    outr, outi = np.empty_like(Ur), np.empty_like(Ui)
    rc = f(M, N, _ptr(Ur), _ptr(Ui), _ptr(Vv), float(s1), float(s2), float(a), float(h2), int(BC),
           int(chunk), float(k), _ptr(outr), _ptr(outi), int(flags))
    if rc != 0:
        raise ValueError("oracle rejected arguments (code %d)" % rc)
    return (outr + 1j * outi).reshape(U.shape, order="F")


def ref_cq2d(U, V, s1, s2, a, h2, BC, chunk, k):
    """The reference's own CQNLSE2D_TAKE_STEPS_2SHOC MEX function (via the shim)."""
    U = np.asarray(U)
    name = "CQNLSE2D_TAKE_STEPS_2SHOC"
    if name not in _refs:
        libs = _build.build_ref()
        if name not in libs:
            raise RuntimeError("reference cubic-quintic integrator is not available here")
        lib = ctypes.CDLL(libs[name], mode=ctypes.RTLD_LOCAL)
        f = lib.mex_call_cq2d
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(ctypes.c_longlong), _dp, _dp, _dp] + \
            [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp]
        _refs[name] = lib
    Ur, Ui, Vv = _planes(U, V)
    cd = (ctypes.c_longlong * 2)(*(int(d) for d in U.shape))
    outr, outi = np.empty_like(Ur), np.empty_like(Ui)
    rc = _refs[name].mex_call_cq2d(cd, _ptr(Ur), _ptr(Ui), _ptr(Vv), float(s1), float(s2),
                                   float(a), float(h2), int(BC), int(chunk), float(k), _ptr(outr),
                                   _ptr(outi))
    if rc != 0:
        raise RuntimeError("reference call failed (code %d)" % rc)
    return (outr + 1j * outi).reshape(U.shape, order="F")
