"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two things are built here, both with plain ``gcc``:

* ``oracle/libnlse_oracle.so`` -- this project's own C restatement of the
  NLSEmagic RK4 chunk integrators (``oracle/nlse_oracle.c``).  It builds on any
  machine and is what the GPU parity tests, ``smoke()`` and the CPU baseline
  leg of ``bench.py`` call.
* ``oracle/_ref/<NAME>.so`` -- the reference's own, unmodified C integrators,
  compiled where they lie under the read-only reference checkout against the
  minimal ``oracle/mexshim`` stand-in for ``mex.h``.  One shared object per
  file, because every file defines ``mexFunction``.  Only possible where the
  reference checkout exists; the outputs are git-ignored.

Compiler flags follow the reference's own Makefile (``-O3 -funroll-loops``,
src_old/NLSE1D_v1/Makefile:6) plus ``-ffp-contract=off`` so that no fused
multiply-add changes the rounding of the reference arithmetic on either x86-64
or aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout: $NLSE_REFERENCE_ROOT, else a sibling directory
# named "reference" next to this checkout.
REFERENCE_ROOT = os.environ.get(
    "NLSE_REFERENCE_ROOT",
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

# name -> path relative to the reference checkout
REF_FILES = {
    "NLSE1D_TAKE_STEPS_CD": "src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c",
    "NLSE1D_TAKE_STEPS_CD_F": "src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD_F.c",
    "NLSE1D_TAKE_STEPS_2SHOC": "src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_2SHOC.c",
    "NLSE1D_TAKE_STEPS_2SHOC_F": "src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_2SHOC_F.c",
    "NLSE2D_TAKE_STEPS_CD": "src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_CD.c",
    "NLSE2D_TAKE_STEPS_CD_F": "src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_CD_F.c",
    "NLSE2D_TAKE_STEPS_2SHOC": "src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_2SHOC.c",
    "NLSE2D_TAKE_STEPS_2SHOC_F": "src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_2SHOC_F.c",
    "NLSE3D_TAKE_STEPS_CD": "src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD.c",
    "NLSE3D_TAKE_STEPS_CD_F": "src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD_F.c",
    "NLSE3D_TAKE_STEPS_2SHOC": "src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC.c",
    "NLSE3D_TAKE_STEPS_2SHOC_F": "src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC_F.c",
    "rmc_vorticity3D": "src/NLSEmagic3D/rmc_vorticity3D.c",
    "CQNLSE2D_TAKE_STEPS_2SHOC": "src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c",
}

REF_CFLAGS = ["-std=gnu89", "-O3", "-funroll-loops", "-ffp-contract=off",
              "-fPIC", "-shared", "-w"]
# -fopenmp: nlse_oracle_set_threads() spreads one solve's grid sweeps over
# threads for the large parity runs (bit-identical; default one thread).
PORT_CFLAGS = ["-std=c99", "-O3", "-funroll-loops", "-ffp-contract=off", "-fopenmp", "-fPIC",
               "-shared", "-Wall", "-Wno-unused-function", "-pthread"]

PORT_SRC = os.path.join(HERE, "nlse_oracle.c")
PORT_LIB = os.path.join(HERE, "libnlse_oracle.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_port(force: bool = False) -> str:
    """Compile this project's C restatement into oracle/libnlse_oracle.so."""
    srcs = [PORT_SRC, os.path.join(HERE, "nlse_oracle_impl.h"), os.path.abspath(__file__)]
    if force or _stale(PORT_LIB, srcs):
        tmp = PORT_LIB + ".tmp%d" % os.getpid()
        _run(["gcc"] + PORT_CFLAGS + [PORT_SRC, "-o", tmp, "-lm"])
        os.replace(tmp, PORT_LIB)
    return PORT_LIB


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE_ROOT, p)) for p in REF_FILES.values())


def build_ref(force: bool = False) -> dict:
    """Compile each reference CPU integrator (unmodified) into oracle/_ref/NAME.so.

    Returns {name: path}.  Returns {} when the reference checkout is absent.
    """
    if not reference_available():
        return {}
    os.makedirs(REF_OUT, exist_ok=True)
    shim_dir = os.path.join(HERE, "mexshim")
    shim_obj = os.path.join(REF_OUT, "mexshim.o")
    if force or _stale(shim_obj, [os.path.join(shim_dir, "mexshim.c"), os.path.join(shim_dir, "mex.h")]):
        _run(["gcc", "-std=c99", "-O2", "-fPIC", "-c", os.path.join(shim_dir, "mexshim.c"),
              "-I", shim_dir, "-o", shim_obj])

    def one(item):
        name, rel = item
        src = os.path.join(REFERENCE_ROOT, rel)
        out = os.path.join(REF_OUT, name + ".so")
        if force or _stale(out, [src, shim_obj]):
            tmp = out + ".tmp%d" % os.getpid()
            _run(["gcc"] + REF_CFLAGS + ["-I", shim_dir, src, shim_obj, "-o", tmp, "-lm"])
            os.replace(tmp, out)
        return name, out

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        return dict(ex.map(one, REF_FILES.items()))


if __name__ == "__main__":
    print(build_port(force="--force" in sys.argv))
    for k, v in build_ref(force="--force" in sys.argv).items():
        print(k, v)
