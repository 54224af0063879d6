"""Python mirror of the NLSEmagic step-function interface, over the C ABI.

Array convention: the MATLAB one.  A grid of MATLAB size M x N x L is a numpy
array of shape (M, N, L) (first index fastest, Fortran order); 2D grids are
(M, N) and 1D grids (M,) (an (M, 1) or (1, M) column/row vector is also taken
as 1D, as the reference does with ``N = mxGetN; if N == 1, N = mxGetM``,
src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:115-118).  Results are new complex128
arrays of the input's shape; inputs are never modified.

Functions:

* ``NLSE{1,2,3}D_TAKE_STEPS_{CD,2SHOC}_CUDA_{D,F}(U, V, s, a, h2, BC,
  chunk_size, k)`` -- the v1 MEX names (e.g.
  src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC_CUDA_D.cu:12-24), double or single
  precision, and ``..._CUDA_M`` for the mixed-precision class.
* ``NLSEmagic{1,2,3}D_Take_Steps_GPU(U, V, s, a, h2, BC, chunk, k,
  precision, method)`` -- the v2 gateways
  (src/NLSEmagic1D/NLSEmagic1D_Take_Steps_GPU.c:33-41); precision 1 single,
  2 double, 3 mixed.
* :class:`Solver` -- the resident-state handle (state and potential stay on
  the GPU between chunks).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import FLAG_MSD_GUARD, PREC_DOUBLE, PREC_MIXED, Problem, check, load

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def grid_dims(shape):
    """(ndim, (M, N, L)) of a MATLAB-shaped array; 1D vectors of either
    orientation are 1D."""
    shape = tuple(int(x) for x in shape)
    if len(shape) == 1:
        return 1, (shape[0], 1, 1)
    if len(shape) == 2 and 1 in shape:
        return 1, (max(shape), 1, 1)
    if len(shape) == 2:
        return 2, (shape[0], shape[1], 1)
    if len(shape) == 3:
        return 3, shape
    raise ValueError("grids must have 1, 2 or 3 dimensions (got shape %s)" % (shape,))


def make_problem(ndim, dims, method, precision, BC, s, a, h2, k, flags=FLAG_MSD_GUARD):
    p = Problem()
    p.ndim = int(ndim)
    for t in range(3):
        p.dims[t] = int(dims[t]) if t < ndim else 1
    p.method = int(method)
    p.precision = int(precision)
    p.bc = int(BC)
    p.s, p.a, p.h2, p.k = float(s), float(a), float(h2), float(k)
    p.flags = int(flags)
    return p


def planar(U):
    """Fortran-order flat real and imaginary planes of U (float64)."""
    U = np.asarray(U)
    re = np.ascontiguousarray(np.real(U).ravel(order="F"), dtype=np.float64)
    im = np.ascontiguousarray(np.imag(U).ravel(order="F") if np.iscomplexobj(U)
                              else np.zeros(U.size), dtype=np.float64)
    return re, im


def take_steps(U, V, s, a, h2, BC, chunk_size, k, method=1, precision=PREC_DOUBLE,
               flags=FLAG_MSD_GUARD):
    """Advance U by chunk_size RK4 steps on the GPU; returns the new U."""
    U = np.asarray(U)
    V = np.asarray(V, dtype=np.float64)
    if V.shape != U.shape:
        raise ValueError("V must have the shape of U (%s vs %s)" % (V.shape, U.shape))
    ndim, dims = grid_dims(U.shape)
    prob = make_problem(ndim, dims, method, precision, BC, s, a, h2, k, flags)
    re, im = planar(U)
    vv = np.ascontiguousarray(V.ravel(order="F"))
    out_r = np.empty_like(re)
    out_i = np.empty_like(im)
    check(load().nlse_take_steps(ctypes.byref(prob), _ptr(re), _ptr(im), _ptr(vv), _ptr(out_r),
                                 _ptr(out_i), int(chunk_size)))
    out = out_r + 1j * out_i
    return out.reshape(U.shape, order="F")


def _legacy(ndim, method, precision):
    def f(U, V, s, a, h2, BC, chunk_size, k):
        got, _ = grid_dims(np.shape(U))
        if got != ndim:
            raise ValueError("this entry point integrates %dD grids (got a %dD array)" % (ndim, got))
        return take_steps(U, V, s, a, h2, BC, chunk_size, k, method=method, precision=precision)

    f.__name__ = "NLSE%dD_TAKE_STEPS_%s_CUDA_%s" % (
        ndim, "CD" if method == 1 else "2SHOC", {1: "F", 2: "D", 3: "M"}[precision])
    f.__doc__ = ("U = %s(U, V, s, a, h2, BC, chunk_size, k): %dD RK4 + %s in %s precision on "
                 "the GPU (drop-in for the NLSEmagic MEX function of that name)."
                 % (f.__name__, ndim, "CD" if method == 1 else "2SHOC",
                    {1: "single", 2: "double", 3: "mixed"}[precision]))
    return f


for _nd in (1, 2, 3):
    for _m in (1, 2):
        for _p in (1, 2, 3):
            _f = _legacy(_nd, _m, _p)
            globals()[_f.__name__] = _f


def _v2(ndim):
    def f(U, V, s, a, h2, BC, chunk, k, precision, method):
        got, _ = grid_dims(np.shape(U))
        if got != ndim:
            raise ValueError("this entry point integrates %dD grids (got a %dD array)" % (ndim, got))
        return take_steps(U, V, s, a, h2, BC, chunk, k, method=method, precision=precision)

    f.__name__ = "NLSEmagic%dD_Take_Steps_GPU" % ndim
    f.__doc__ = ("U = %s(U, V, s, a, h2, BC, chunk, k, precision, method) (precision 1 single, "
                 "2 double, 3 mixed; method 1 CD, 2 2SHOC)." % f.__name__)
    return f


NLSEmagic1D_Take_Steps_GPU = _v2(1)
NLSEmagic2D_Take_Steps_GPU = _v2(2)
NLSEmagic3D_Take_Steps_GPU = _v2(3)


def linear_stability_k(ndim, method, h, a):
    return load().nlse_linear_stability_k(int(ndim), int(method), float(h), float(a))


class Solver:
    """Resident solve: state and potential live on the current CUDA device.

    ``shape`` is the MATLAB-shaped grid shape.  All work is enqueued on the
    solver's own stream (``self.stream``, a cudaStream_t handle)."""

    def __init__(self, shape, method=2, precision=PREC_MIXED, BC=1, s=-1.0, a=1.0, h2=0.01,
                 k=1e-3, flags=FLAG_MSD_GUARD):
        self.shape = tuple(int(x) for x in shape)
        self.ndim, self.dims = grid_dims(self.shape)
        self.n = int(np.prod(self.shape))
        self.problem = make_problem(self.ndim, self.dims, method, precision, BC, s, a, h2, k, flags)
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.nlse_solver_create(ctypes.byref(self.problem), ctypes.byref(h)))
        self._h = h

    # -- initial conditions and diagnostics on the device
    @staticmethod
    def _ic(kind, items=None, om=0.0, c=0.0, x0=0.0, omega=0.0, noise_kind=_lib.NOISE_NONE,
            noise=0.0, seed=0):
        ic = _lib.InitialCondition()
        ic.kind = int(kind)
        arr = None
        if items is not None:
            arr = np.ascontiguousarray(np.asarray(items, dtype=np.float64).ravel())
            ic.items = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            ic.count = int(arr.size // (3 if kind == _lib.IC_VORTICES else 7))
        ic.om, ic.c, ic.x0, ic.omega = float(om), float(c), float(x0), float(omega)
        ic.noise_kind, ic.noise, ic.seed = int(noise_kind), float(noise), int(seed)
        return ic, arr

    def init_ic(self, kind, items=None, **kw):
        """Generate the initial state and potential on the device.  kind:
        IC_SECH, IC_TANH, IC_GAUSS, IC_GREY (1D; om, c, x0), IC_VORTICES (2D;
        items = [(x, y, charge), ...]), IC_RINGS (3D; items = [(cx, cy, cz, nx,
        ny, nz, radius), ...], omega = trap frequency); optional noise_kind
        (NOISE_ADD / NOISE_PHASE), noise, seed."""
        ic, keep = self._ic(kind, items, **kw)
        check(self._lib.nlse_solver_init_ic(self._h, ctypes.byref(ic)))
        del keep

    def diagnostics(self):
        """dict(mass = sum |psi|^2 h^d, max_abs2, max_re, nonfinite), reduced on the device."""
        d = _lib.Diagnostics()
        check(self._lib.nlse_solver_diagnostics(self._h, ctypes.byref(d)))
        return {"mass": d.mass, "max_abs2": d.max_abs2, "max_re": d.max_re,
                "nonfinite": int(d.nonfinite)}

    def error_1d(self, kind, t, **kw):
        """Maximum errors (Re, Im, |psi|^2) against the closed-form 1D soliton at time t."""
        ic, keep = self._ic(kind, **kw)
        err = (ctypes.c_double * 3)()
        check(self._lib.nlse_solver_error_1d(self._h, ctypes.byref(ic), float(t), err))
        del keep
        return tuple(err)

    def vorticity(self, veps=1e-10):
        """Vorticity (wx, wy, wz, W) of the current 3D state, computed on the
        device from the resident state; returned as numpy arrays of the grid
        shape (the device buffers come from torch, used only as an
        allocator)."""
        import torch
        if self.ndim != 3:
            raise ValueError("vorticity needs a 3D solve")
        bufs = [torch.empty(self.n, dtype=torch.float64, device="cuda") for _ in range(4)]
        check(self._lib.nlse_solver_vorticity(self._h, float(veps),
                                              *(ctypes.c_void_p(b.data_ptr()) for b in bufs)))
        self.sync()
        return tuple(b.cpu().numpy().reshape(self.shape, order="F") for b in bufs)

    @staticmethod
    def bytes_for(shape, method=2, precision=PREC_MIXED, BC=1, flags=FLAG_MSD_GUARD):
        """Device bytes a solver of this shape and class holds after a host upload."""
        ndim, dims = grid_dims(shape)
        p = make_problem(ndim, dims, method, precision, BC, 0.0, 1.0, 1.0, 1.0, flags)
        return int(load().nlse_solver_bytes_for(ctypes.byref(p)))

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._lib.nlse_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- data movement
    def upload(self, U, V):
        re, im = planar(U)
        vv = np.ascontiguousarray(np.asarray(V, dtype=np.float64).ravel(order="F"))
        if re.size != self.n or vv.size != self.n:
            raise ValueError("U and V must have %d points" % self.n)
        check(self._lib.nlse_solver_upload(self._h, _ptr(re), _ptr(im), _ptr(vv)))

    def upload_device(self, re_ptr, im_ptr, v_ptr):
        """Device pointers (ints) to planar float64 arrays of n points."""
        check(self._lib.nlse_solver_upload_device(self._h, ctypes.c_void_p(re_ptr),
                                                  ctypes.c_void_p(im_ptr), ctypes.c_void_p(v_ptr)))

    def download(self):
        re = np.empty(self.n)
        im = np.empty(self.n)
        check(self._lib.nlse_solver_download(self._h, _ptr(re), _ptr(im)))
        return (re + 1j * im).reshape(self.shape, order="F")

    def download_device(self, re_ptr, im_ptr):
        check(self._lib.nlse_solver_download_device(self._h, ctypes.c_void_p(re_ptr),
                                                    ctypes.c_void_p(im_ptr)))

    # -- stepping
    def run(self, nsteps):
        check(self._lib.nlse_solver_run(self._h, int(nsteps)))

    def sync(self):
        check(self._lib.nlse_solver_sync(self._h))

    def idle(self):
        """True when the queued steps have finished (non-blocking)."""
        out = ctypes.c_int()
        check(self._lib.nlse_solver_query(self._h, ctypes.byref(out)))
        return bool(out.value)

    def sum_abs2(self):
        """sum over points of |U|^2, accumulated in FP64 (multiply by h^d for
        the mass)."""
        out = ctypes.c_double()
        check(self._lib.nlse_solver_mass(self._h, ctypes.byref(out)))
        return out.value

    def set_graph_steps(self, steps):
        check(self._lib.nlse_solver_set_graph_steps(self._h, int(steps)))

    @property
    def stream(self) -> int:
        st = ctypes.c_void_p()
        check(self._lib.nlse_solver_stream(self._h, ctypes.byref(st)))
        return st.value or 0

    @property
    def launches_per_step(self) -> int:
        return int(self._lib.nlse_solver_launches_per_step(self._h))

    @property
    def device_bytes(self) -> int:
        return int(self._lib.nlse_solver_device_bytes(self._h))


class Batch:
    """Many independent solves advancing together in one persistent launch
    per :meth:`run` call (FP64 and mixed precision classes may be mixed).

    ``pool_bytes`` is the device memory budget for solve state; :meth:`add`
    raises :class:`~nlsemagic_gb300._lib.NLSEError` with code
    NLSE_ERR_CAPACITY when a solve does not fit."""

    def __init__(self, pool_bytes, max_solves=4096):
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.nlse_batch_create(int(pool_bytes), int(max_solves), ctypes.byref(h)))
        self._h = h
        self.shapes = {}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nlse_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def bytes_for(shape, precision, method=2):
        """Pool bytes one solve takes (2SHOC solves also hold their D scratch)."""
        ndim, dims = grid_dims(shape)
        p = make_problem(ndim, dims, method, precision, 1, 0.0, 1.0, 1.0, 1.0)
        return int(load().nlse_batch_bytes_for(ctypes.byref(p)))

    def add(self, U, V, s, a, h2, BC, nsteps, k, method=2, precision=PREC_MIXED,
            flags=FLAG_MSD_GUARD):
        U = np.asarray(U)
        ndim, dims = grid_dims(U.shape)
        p = make_problem(ndim, dims, method, precision, BC, s, a, h2, k, flags)
        re, im = planar(U)
        vv = np.ascontiguousarray(np.asarray(V, dtype=np.float64).ravel(order="F"))
        slot = ctypes.c_int()
        check(self._lib.nlse_batch_add(self._h, ctypes.byref(p), _ptr(re), _ptr(im), _ptr(vv),
                                       int(nsteps), ctypes.byref(slot)))
        self.shapes[slot.value] = U.shape
        return slot.value

    def run(self, max_steps):
        check(self._lib.nlse_batch_run(self._h, int(max_steps)))

    def sync(self):
        check(self._lib.nlse_batch_sync(self._h))

    def idle(self):
        """True when the queued launches have finished (non-blocking)."""
        out = ctypes.c_int()
        check(self._lib.nlse_batch_query(self._h, ctypes.byref(out)))
        return bool(out.value)

    def remaining(self, slot):
        out = ctypes.c_longlong()
        check(self._lib.nlse_batch_remaining(self._h, int(slot), ctypes.byref(out)))
        return out.value

    def download(self, slot):
        shape = self.shapes[slot]
        n = int(np.prod(shape))
        re = np.empty(n)
        im = np.empty(n)
        check(self._lib.nlse_batch_download(self._h, int(slot), _ptr(re), _ptr(im)))
        return (re + 1j * im).reshape(shape, order="F")

    def remove(self, slot):
        check(self._lib.nlse_batch_remove(self._h, int(slot)))
        self.shapes.pop(slot, None)

    def stats(self):
        a = ctypes.c_int()
        pts = ctypes.c_longlong()
        free = ctypes.c_longlong()
        check(self._lib.nlse_batch_stats(self._h, ctypes.byref(a), ctypes.byref(pts),
                                         ctypes.byref(free)))
        return {"active": a.value, "points": pts.value, "free_bytes": free.value}

    @property
    def stream(self):
        st = ctypes.c_void_p()
        check(self._lib.nlse_batch_stream(self._h, ctypes.byref(st)))
        return st.value or 0

    @property
    def last_launches(self):
        return int(self._lib.nlse_batch_last_launches(self._h))


# ---------------------------------------------------------------------------
# 3D vorticity (post-chunk analysis)
# ---------------------------------------------------------------------------
def rmc_vorticity3D(U, lh2, veps):
    """[w_x, w_y, w_z, W] = rmc_vorticity3D(U, 1/(h*2), veps) on the GPU
    (src/NLSEmagic3D/rmc_vorticity3D.c:12-16): U MATLAB-shaped (M, N, L),
    complex or real.  Returns four real arrays of U's shape."""
    U = np.asarray(U)
    if U.ndim != 3:
        raise ValueError("rmc_vorticity3D needs a 3D array")
    re = np.ascontiguousarray(np.real(U).ravel(order="F"), dtype=np.float64)
    im = (np.ascontiguousarray(np.imag(U).ravel(order="F"), dtype=np.float64)
          if np.iscomplexobj(U) else None)
    dims = (ctypes.c_longlong * 3)(*(int(d) for d in U.shape))
    outs = [np.empty(U.size) for _ in range(4)]
    check(load().nlse_vorticity3d(_ptr(re), _ptr(im) if im is not None else None, dims,
                                  float(lh2), float(veps), *(_ptr(o) for o in outs)))
    return tuple(o.reshape(U.shape, order="F") for o in outs)


def vorticity3d(U, h, veps=1e-10):
    """Vorticity of U on a grid of spacing h: rmc_vorticity3D(U, 1/(2h), veps)."""
    return rmc_vorticity3D(U, 1.0 / (2.0 * h), veps)


# ---------------------------------------------------------------------------
# 2D cubic-quintic NLSE (2SHOC, FP64)
# ---------------------------------------------------------------------------
def CQNLSE2D_TAKE_STEPS_2SHOC(U, V, s1, s2, a, h2, BC, chunk_size, k, flags=FLAG_MSD_GUARD):
    """U = CQNLSE2D_TAKE_STEPS_2SHOC(U, V, s1, s2, a, h2, BC, chunk_size, k) on
    the GPU (src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c:357-437); U
    MATLAB-shaped (M, N)."""
    U = np.asarray(U)
    if U.ndim != 2:
        raise ValueError("the cubic-quintic integrator is 2D")
    ndim, dims = grid_dims(U.shape)
    prob = make_problem(2, dims, 2, PREC_DOUBLE, BC, s1, a, h2, k, flags)
    re, im = planar(U)
    vv = np.ascontiguousarray(np.asarray(V, dtype=np.float64).ravel(order="F"))
    outr, outi = np.empty_like(re), np.empty_like(im)
    check(load().nlse_cq2d_take_steps(ctypes.byref(prob), float(s2), _ptr(re), _ptr(im),
                                      _ptr(vv), _ptr(outr), _ptr(outi), int(chunk_size)))
    return (outr + 1j * outi).reshape(U.shape, order="F")
