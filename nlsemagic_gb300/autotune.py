"""Autotuner for the stage-kernel launch configuration.

For one problem class (dimension, grid, method, precision, boundary code) it
times RK4 steps of a resident :class:`~nlsemagic_gb300.api.Solver` on a
smooth synthetic state for each candidate setting of the library's tuning
knobs and keeps the fastest:

* ``wide.zc``      z-chunk length of the mixed-precision 3D kernel (planes a
                   CTA streams through; trades queue-fill overhead against the
                   number of CTAs in flight; 0: the library's choice),
* ``wide.ty``      tile height of that kernel (4, 8 or 16 rows of 32 columns:
                   halo re-reads against CTAs in flight),
* ``graph.steps``  RK4 steps captured per CUDA graph (launch overhead against
                   graph size; matters for small grids),
* ``wide2d.ty``    tile height of the mixed-precision 2D stage kernel (8, 16
                   or 32 rows: CTAs in flight against halo re-reads).

The library has more knobs that give the same bits either way and are not
tuned here, among them ``wide.pdl`` (1 by default: the 3D 2SHOC stage
kernels are launched with programmatic dependent launch; 0: plain stream
order) and ``wide.strips`` (1 by default: the 3D 2SHOC face kernels take the
x faces' own lo, K and V from face-indexed arrays).

Results are cached in a JSON file (``$NLSE_TUNE_CACHE`` or
``~/.cache/nlse_gb300/tune.json``) keyed by device name and problem class;
:func:`apply` sets the knobs from the cache before a workload runs.  The
knobs are process-wide and are read when a stage launch is issued or a graph
captured, so they apply to solvers created afterwards.
"""
from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from . import _lib
from .api import Solver, grid_dims

KNOBS = ("wide.zc", "wide.ty", "graph.steps", "wide2d.ty")


def set_knob(key, value):
    _lib.check(_lib.load().nlse_tune_set(key.encode(), int(value)))


def get_knob(key):
    v = ctypes.c_longlong()
    _lib.check(_lib.load().nlse_tune_get(key.encode(), ctypes.byref(v)))
    return v.value


def cache_path():
    return os.environ.get("NLSE_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "nlse_gb300",
                                       "tune.json"))


def _device_name():
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "cuda"


def problem_key(shape, method, precision, BC):
    ndim, dims = grid_dims(shape)
    return "%s|%dd|%s|m%d|p%d|bc%d" % (_device_name(), ndim, "x".join(str(d) for d in shape),
                                       method, precision, BC)


def _load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_cache(c):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(c, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _smooth_state(shape, h):
    axes = [np.arange(n) * h - n * h / 2 for n in shape]
    grids = np.meshgrid(*axes, indexing="ij")
    r2 = sum(g * g for g in grids)
    U = (np.tanh(np.sqrt(r2) + 0.5) * np.exp(1j * 0.1 * grids[0])).astype(np.complex128)
    return U, 0.5 * r2 / max(r2.max(), 1e-30)


def candidates(shape, precision):
    ndim, dims = grid_dims(shape)
    cands = []
    zcs, wtys, tys = [0], [8], [0]
    if ndim == 3 and precision == 3:
        L = dims[2]
        zcs = [0] + sorted({z for z in (16, 32, 64) if 4 <= z <= L})
        wtys = [4, 8, 16]
    if ndim == 2 and precision == 3:
        tys = [8, 16, 32]
    for zc in zcs:
        for wty in wtys:
            for ty in tys:
                for gs in (4, 10, 25):
                    cands.append({"wide.zc": zc, "wide.ty": wty, "graph.steps": gs,
                                  "wide2d.ty": ty})
    return cands


def _solver_for(shape, method, precision, BC, h=0.3):
    U, V = _smooth_state(shape, h)
    ndim, _ = grid_dims(shape)
    from .workloads import linear_stability_k
    k = 0.5 * linear_stability_k(ndim, method, h, 1.0)
    sv = Solver(shape, method=method, precision=precision, BC=BC, s=-1.0, a=1.0, h2=h * h, k=k)
    sv.upload(U, V)
    return sv


def time_config(shape, method, precision, BC, cfg, steps, reps=2, solver=None):
    """Best of reps timings of `steps` RK4 steps with the knobs of cfg.  A
    given solver is reused: its graphs are captured again under cfg (the
    knobs are read at capture; none of them changes what the solver
    allocates)."""
    for k, v in cfg.items():
        set_knob(k, v)
    own = solver is None
    s = _solver_for(shape, method, precision, BC) if own else solver
    try:
        gs = max(1, cfg.get("graph.steps", 8))
        s.set_graph_steps(0)   # drop the graphs captured under other knobs
        s.set_graph_steps(gs)
        s.run(gs)  # capture outside the timing
        s.sync()
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            s.run(steps)
            s.sync()
            best = min(best, time.perf_counter() - t0)
    finally:
        if own:
            s.close()
    return best


def tune(shape, method=2, precision=3, BC=2, steps=20, force=False, verbose=False):
    """Time every candidate (one solver, its graphs captured again for each),
    cache and return the best configuration."""
    key = problem_key(shape, method, precision, BC)
    cache = _load_cache()
    if key in cache and not force:
        return cache[key]
    saved = {k: get_knob(k) for k in KNOBS}
    results = []
    sv = _solver_for(shape, method, precision, BC)
    try:
        for cfg in candidates(shape, precision):
            t = time_config(shape, method, precision, BC, cfg, steps, solver=sv)
            results.append((t, cfg))
            if verbose:
                print("%-40s %.4f s" % (cfg, t))
    finally:
        sv.close()
        for k, v in saved.items():
            set_knob(k, v)
    t, best = min(results, key=lambda r: r[0])
    n = int(np.prod(shape))
    entry = dict(best, seconds_per_step=t / steps, gpt_steps_per_s=n * steps / t / 1e9,
                 candidates=len(results))
    cache[key] = entry
    _save_cache(cache)
    return entry


def apply(shape, method=2, precision=3, BC=2):
    """Set the knobs from the cache for this problem class; returns the entry
    used (or None when the class was never tuned)."""
    entry = _load_cache().get(problem_key(shape, method, precision, BC))
    if entry:
        for k in KNOBS:
            if k in entry:
                set_knob(k, entry[k])
    return entry
