"""The C-ABI library loads and exports every symbol include/*.h declares;
argument validation happens before any CUDA call (so it is testable here)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import nlsemagic_gb300 as ng
from nlsemagic_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"^\s*#[^\n]*", "", src, flags=re.M)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{]*?)\)\s*;", src):
            name = m.group(1)
            if name in ("if", "while", "for", "return", "sizeof"):
                continue
            names.append(name)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from nlsemagic_gb300 import build
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("NLSE1D_TAKE_STEPS_CUDA", "NLSE3D_TAKE_STEPS_CUDA_F", "nlse_take_steps",
                 "nlse_solver_create", "nlse_solver_run", "nlse_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header(lib):
    # every declared symbol has a ctypes signature (so no call goes untyped)
    missing = set(declared_functions()) - set(_lib.SIGNATURES)
    assert not missing, missing


def test_tuning_knobs_roundtrip_and_validation(lib):
    from nlsemagic_gb300 import autotune
    old = autotune.get_knob("wide.zc")
    autotune.set_knob("wide.zc", 48)
    assert autotune.get_knob("wide.zc") == 48
    autotune.set_knob("wide.zc", old)
    with pytest.raises(_lib.NLSEError):
        autotune.set_knob("no.such.knob", 1)
    with pytest.raises(_lib.NLSEError):
        autotune.set_knob("graph.steps", -3)
    for key, good, bad in (("wide2d", 0, 2), ("wide2d.ty", 16, 12), ("seg1d", 0, 2),
                           ("io.zero_copy", 0, 3)):
        old = autotune.get_knob(key)
        autotune.set_knob(key, good)
        assert autotune.get_knob(key) == good
        with pytest.raises(_lib.NLSEError):
            autotune.set_knob(key, bad)
        autotune.set_knob(key, old)


def test_single_pass_2d_needs_no_d_scratch(lib):
    # 2D 2SHOC on the single-pass kernels (mixed, FP32) allocates no D
    # scratch: 8 bytes a point less than with the gather kernels
    from nlsemagic_gb300 import autotune
    shape, n = (300, 200), 300 * 200
    old = autotune.get_knob("wide2d")
    try:
        for prec in (ng.PREC_MIXED, ng.PREC_SINGLE):
            autotune.set_knob("wide2d", 1)
            on = ng.Solver.bytes_for(shape, method=2, precision=prec, BC=1)
            autotune.set_knob("wide2d", 0)
            off = ng.Solver.bytes_for(shape, method=2, precision=prec, BC=1)
            assert off - on == 8 * n, (prec, on, off)
        autotune.set_knob("wide2d", 1)  # FP64 keeps the two-launch form and its scratch
        a = ng.Solver.bytes_for(shape, method=2, precision=ng.PREC_DOUBLE, BC=1)
        autotune.set_knob("wide2d", 0)
        assert ng.Solver.bytes_for(shape, method=2, precision=ng.PREC_DOUBLE, BC=1) == a
    finally:
        autotune.set_knob("wide2d", old)


def test_bytes_for_counts_the_x_face_strips(lib):
    # a 3D 2SHOC mixed solver keeps five face-indexed strip arrays of 2 N L
    # entries (lo twice and K as float2, V twice as float); the estimate the
    # serving loop admits by includes them
    shape = (40, 30, 20)
    M, N, L = shape
    mixed = ng.Solver.bytes_for(shape, method=2, precision=ng.PREC_MIXED, BC=2)
    cd = ng.Solver.bytes_for(shape, method=1, precision=ng.PREC_MIXED, BC=2)
    n = M * N * L
    ghosts = mixed - cd - 8 * n - (3 * 8 + 2 * 4) * 2 * N * L  # ghost and F scratch remain
    assert ghosts > 0 and ghosts % 16 == 0, (mixed, cd)


def test_autotune_candidates_per_class():
    from nlsemagic_gb300 import autotune
    two = autotune.candidates((256, 256), 3)
    assert {c["wide2d.ty"] for c in two} == {8, 16, 32}
    assert all(c["wide.zc"] == 0 for c in two)
    three = autotune.candidates((64, 64, 64), 3)
    assert {c["wide2d.ty"] for c in three} == {0} and len({c["wide.zc"] for c in three}) > 1
    assert {c["wide.ty"] for c in three} == {4, 8, 16}
    assert {c["wide.ty"] for c in two} == {8}
    assert all(set(c) == set(autotune.KNOBS) for c in two + three)


def _call(lib, U, BC=2, method=1, precision=2, dims=None, h2=0.01, k=1e-3, chunk=1):
    re_, im_ = ng.api.planar(U)
    V = np.zeros(re_.size)
    ndim, d = ng.api.grid_dims(U.shape)
    p = ng.api.make_problem(ndim, dims or d, method, precision, BC, -1.0, 1.0, h2, k)
    outr = np.empty_like(re_)
    outi = np.empty_like(im_)
    dp = ctypes.POINTER(ctypes.c_double)
    return lib.nlse_take_steps(ctypes.byref(p), re_.ctypes.data_as(dp), im_.ctypes.data_as(dp),
                               V.ctypes.data_as(dp), outr.ctypes.data_as(dp),
                               outi.ctypes.data_as(dp), chunk)


@pytest.mark.parametrize("kw,why", [
    (dict(U=np.ones(2, complex)), "too few points"),
    (dict(U=np.ones((3, 3), complex), BC=4), "BC 4 is 1D only"),
    (dict(U=np.ones(8, complex), BC=7), "unknown BC"),
    (dict(U=np.ones(8, complex), method=3), "unknown method"),
    (dict(U=np.ones(8, complex), precision=9), "unknown precision"),
    (dict(U=np.ones(8, complex), h2=0.0), "h2 must be > 0"),
    (dict(U=np.ones(8, complex), k=-1.0), "k must be > 0"),
    (dict(U=np.ones(8, complex), chunk=-1), "negative chunk"),
])
def test_invalid_arguments_rejected_before_cuda(lib, kw, why):
    rc = _call(lib, **kw)
    assert rc == _lib.NLSE_ERR_ARG, why
    assert _lib.last_error()


def test_contracted_flag_is_fp64_only(lib):
    # NLSE_FLAG_FMA asks for the FP64 kernels compiled with contraction; other
    # classes reject it before any CUDA call
    re_, im_ = ng.api.planar(np.ones(16, complex))
    V = np.zeros(16)
    dp = ctypes.POINTER(ctypes.c_double)
    out = [np.empty(16), np.empty(16)]
    for prec in (1, 3):
        p = ng.api.make_problem(1, (16, 1, 1), 1, prec, 1, -1.0, 1.0, 0.01, 1e-3,
                                ng.FLAG_MSD_GUARD | ng.FLAG_FMA)
        rc = lib.nlse_take_steps(ctypes.byref(p), re_.ctypes.data_as(dp), im_.ctypes.data_as(dp),
                                 V.ctypes.data_as(dp), out[0].ctypes.data_as(dp),
                                 out[1].ctypes.data_as(dp), 1)
        assert rc == ng._lib.NLSE_ERR_ARG
        assert b"FP64 class only" in lib.nlse_last_error_string()


def test_stability_helper(lib):
    k = ng.linear_stability_k(3, 2, 0.3, 1.0)
    assert abs(k - 0.75 * 0.09 / (3 * 2 ** 0.5)) < 1e-15


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(_lib.NativeLibraryMissing):
        saved = _lib._lib
        try:
            _lib._lib = None
            _lib.load(str(tmp_path / "absent.so"))
        finally:
            _lib._lib = saved


def test_ctypes_structs_match_the_c_header(tmp_path):
    # sizes and field offsets of the structures passed by pointer
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "nlse_gb300.h"\n'
        'int main(void){\n'
        ' printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(nlse_problem), offsetof(nlse_problem,dims),'
        ' offsetof(nlse_problem,s), offsetof(nlse_problem,flags), sizeof(nlse_ic), offsetof(nlse_ic,items),'
        ' offsetof(nlse_ic,seed));\n'
        ' printf("%zu %zu %zu\\n", sizeof(nlse_diag), offsetof(nlse_diag,max_re), offsetof(nlse_diag,nonfinite));\n'
        ' return 0;}\n')
    exe = tmp_path / "layout"
    import subprocess
    r = subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()
    want = [ctypes.sizeof(_lib.Problem), _lib.Problem.dims.offset, _lib.Problem.s.offset,
            _lib.Problem.flags.offset, ctypes.sizeof(_lib.InitialCondition),
            _lib.InitialCondition.items.offset, _lib.InitialCondition.seed.offset,
            ctypes.sizeof(_lib.Diagnostics), _lib.Diagnostics.max_re.offset,
            _lib.Diagnostics.nonfinite.offset]
    assert [int(v) for v in out] == want
