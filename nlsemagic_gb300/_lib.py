"""ctypes binding of libnlse_gb300.so (the C ABI of include/nlse_gb300.h).

The shared library is loaded from this package directory.  There is no CPU
fallback: if the library is missing, every entry point raises
:class:`NativeLibraryMissing`.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnlse_gb300.so")

NLSE_OK = 0
NLSE_ERR_ARG = 1
NLSE_ERR_CUDA = 2
NLSE_ERR_NOMEM = 3
NLSE_ERR_TIMEOUT = 4
NLSE_ERR_NONFINITE = 5
NLSE_ERR_CAPACITY = 6
NLSE_ERR_STATE = 7

PREC_SINGLE, PREC_DOUBLE, PREC_MIXED = 1, 2, 3
FLAG_MSD_GUARD = 1
FLAG_GATHER = 2
FLAG_FMA = 4

_ERRNAMES = {1: "NLSE_ERR_ARG", 2: "NLSE_ERR_CUDA", 3: "NLSE_ERR_NOMEM", 4: "NLSE_ERR_TIMEOUT",
             5: "NLSE_ERR_NONFINITE", 6: "NLSE_ERR_CAPACITY", 7: "NLSE_ERR_STATE"}


class NativeLibraryMissing(RuntimeError):
    pass


class NLSEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (_ERRNAMES.get(code, "error %d" % code), msg))
        self.code = code


class Problem(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("dims", ctypes.c_longlong * 3), ("method", ctypes.c_int),
                ("precision", ctypes.c_int), ("bc", ctypes.c_int), ("s", ctypes.c_double),
                ("a", ctypes.c_double), ("h2", ctypes.c_double), ("k", ctypes.c_double),
                ("flags", ctypes.c_int)]


IC_SECH, IC_TANH, IC_GAUSS, IC_GREY, IC_VORTICES, IC_RINGS = 1, 2, 3, 4, 5, 6
NOISE_NONE, NOISE_ADD, NOISE_PHASE = 0, 1, 2


class InitialCondition(ctypes.Structure):
    """nlse_ic of include/nlse_gb300.h."""
    _fields_ = [("kind", ctypes.c_int), ("count", ctypes.c_int),
                ("items", ctypes.POINTER(ctypes.c_double)), ("om", ctypes.c_double),
                ("c", ctypes.c_double), ("x0", ctypes.c_double), ("omega", ctypes.c_double),
                ("noise_kind", ctypes.c_int), ("noise", ctypes.c_double),
                ("seed", ctypes.c_ulonglong)]


class Diagnostics(ctypes.Structure):
    """nlse_diag of include/nlse_gb300.h."""
    _fields_ = [("mass", ctypes.c_double), ("max_abs2", ctypes.c_double),
                ("max_re", ctypes.c_double), ("nonfinite", ctypes.c_longlong)]


_lib = None
_lock = threading.Lock()
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p
_i, _d, _ll = ctypes.c_int, ctypes.c_double, ctypes.c_longlong

# name -> (restype, argtypes)
SIGNATURES = {
    "nlse_last_error_string": (ctypes.c_char_p, []),
    "nlse_version": (ctypes.c_char_p, []),
    "nlse_linear_stability_k": (_d, [_i, _i, _d, _d]),
    "nlse_take_steps": (_i, [ctypes.POINTER(Problem), _dp, _dp, _dp, _dp, _dp, _i]),
    "nlse_solver_create": (_i, [ctypes.POINTER(Problem), ctypes.POINTER(_vp)]),
    "nlse_solver_destroy": (_i, [_vp]),
    "nlse_solver_upload": (_i, [_vp, _dp, _dp, _dp]),
    "nlse_solver_upload_device": (_i, [_vp, _vp, _vp, _vp]),
    "nlse_solver_run": (_i, [_vp, _ll]),
    "nlse_solver_download": (_i, [_vp, _dp, _dp]),
    "nlse_solver_download_device": (_i, [_vp, _vp, _vp]),
    "nlse_solver_mass": (_i, [_vp, _dp]),
    "nlse_solver_sync": (_i, [_vp]),
    "nlse_solver_query": (_i, [_vp, ctypes.POINTER(_i)]),
    "nlse_solver_stream": (_i, [_vp, ctypes.POINTER(_vp)]),
    "nlse_solver_set_graph_steps": (_i, [_vp, _i]),
    "nlse_solver_launches_per_step": (_i, [_vp]),
    "nlse_solver_device_bytes": (_ll, [_vp]),
    "nlse_solver_bytes_for": (_ll, [ctypes.POINTER(Problem)]),
    "nlse_vorticity3d": (_i, [_dp, _dp, ctypes.POINTER(_ll), ctypes.c_double, ctypes.c_double,
                              _dp, _dp, _dp, _dp]),
    "nlse_solver_vorticity": (_i, [_vp, ctypes.c_double, _vp, _vp, _vp, _vp]),
    "nlse_solver_init_ic": (_i, [_vp, ctypes.POINTER(InitialCondition)]),
    "nlse_cq2d_take_steps": (_i, [ctypes.POINTER(Problem), ctypes.c_double, _dp, _dp, _dp, _dp,
                                  _dp, _i]),
    "nlse_solver_diagnostics": (_i, [_vp, ctypes.POINTER(Diagnostics)]),
    "nlse_solver_error_1d": (_i, [_vp, ctypes.POINTER(InitialCondition), ctypes.c_double, _dp]),
    "nlse_batch_create": (_i, [_ll, _i, ctypes.POINTER(_vp)]),
    "nlse_batch_destroy": (_i, [_vp]),
    "nlse_batch_bytes_for": (_ll, [ctypes.POINTER(Problem)]),
    "nlse_batch_add": (_i, [_vp, ctypes.POINTER(Problem), _dp, _dp, _dp, _ll,
                            ctypes.POINTER(_i)]),
    "nlse_batch_run": (_i, [_vp, _i]),
    "nlse_batch_remaining": (_i, [_vp, _i, ctypes.POINTER(_ll)]),
    "nlse_batch_download": (_i, [_vp, _i, _dp, _dp]),
    "nlse_batch_remove": (_i, [_vp, _i]),
    "nlse_batch_sync": (_i, [_vp]),
    "nlse_batch_query": (_i, [_vp, ctypes.POINTER(_i)]),
    "nlse_batch_stats": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_ll), ctypes.POINTER(_ll)]),
    "nlse_batch_stream": (_i, [_vp, ctypes.POINTER(_vp)]),
    "nlse_batch_last_launches": (_i, [_vp]),
    "nlse_take_steps_noalloc": (_i, [ctypes.POINTER(Problem), _vp, _vp, _vp, _vp, _vp, _i,
                                     _vp]),
    "nlse_device_fp64_rates": (_i, [_dp, _dp]),
    "nlse_tune_set": (_i, [ctypes.c_char_p, _ll]),
    "nlse_tune_get": (_i, [ctypes.c_char_p, ctypes.POINTER(_ll)]),
}
for _dim, _dims in ((1, [_i]), (2, [_i, _i]), (3, [_i, _i, _i])):
    SIGNATURES["NLSE%dD_TAKE_STEPS_CUDA" % _dim] = (
        _i, [_dp, _dp, _dp, _dp, _dp, _d, _d, _d, _i, _i, _d] + _dims + [_i])
    SIGNATURES["NLSE%dD_TAKE_STEPS_CUDA_MIXED" % _dim] = (
        _i, [_dp, _dp, _dp, _dp, _dp, _d, _d, _d, _i, _i, _d] + _dims + [_i])
    SIGNATURES["NLSE%dD_TAKE_STEPS_CUDA_F" % _dim] = (
        _i, [_fp, _fp, _fp, _fp, _fp, ctypes.c_float, ctypes.c_float, ctypes.c_float, _i, _i,
             ctypes.c_float] + _dims + [_i])


def load(path: str = LIB_PATH):
    """Load the shared library (once) and declare every exported symbol."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise NativeLibraryMissing(
                "libnlse_gb300.so is not built (expected at %s); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` or "
                "`python nlsemagic_gb300/build.py`" % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    return load().nlse_last_error_string().decode(errors="replace")


def check(rc: int):
    if rc != NLSE_OK:
        raise NLSEError(rc, last_error())
    return rc
