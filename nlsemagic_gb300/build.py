"""Build the CUDA library libnlse_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel to an object file under
``nlsemagic_gb300/_build/`` and the objects are linked into
``nlsemagic_gb300/libnlse_gb300.so``.  The exact-precision unit is compiled
with ``-fmad=false`` so that no multiply-add is contracted (bit-identical
FP64 / FP32 results against the reference C integrators); host code is
compiled with ``-ffp-contract=off`` for the same reason on aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnlse_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE]

# unit -> extra flags
UNITS = {
    "kern_exact.cu": ["-fmad=false"],
    "kern_mixed.cu": [],
    "kern_util.cu": [],
    "nlse_abi.cu": [],
    "nlse_batch.cu": ["-fmad=false"],
    "nlse_noalloc.cu": [],
    "kern_vort.cu": ["-fmad=false"],
    "kern_init.cu": [],
    "kern_cq.cu": ["-fmad=false"],
    "kern_small_exact.cu": ["-fmad=false"],
    "kern_small_mixed.cu": [],
    "kern_probe.cu": [],
    "kern_exact_fma.cu": [],  # contracted FP64 (NLSE_FLAG_FMA): -fmad left on
    "nlse_batch_fma.cu": [],  # the batched launch's contracted FP64 kernel
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build nlsemagic_gb300")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
           [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    # extra nvcc flags (e.g. -DNLSE_WIDE_MIN_BLOCKS=4); a change forces a rebuild
    extra = os.environ.get("NLSE_NVCC_FLAGS", "").split()
    stamp = os.path.join(BUILD, "flags.txt")
    old_flags = open(stamp).read() if os.path.exists(stamp) else ""
    if old_flags != " ".join(extra):
        force = True
        if os.path.exists(stamp):
            os.remove(stamp)
    objs = []

    def compile_one(u):
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        if force or ptxas_info or _stale(obj, [src, __file__] + hdrs):
            cmd = [nv] + ARCH + COMMON + UNITS[u] + extra + \
                  (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj + ".tmp"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (u, " ".join(cmd), r.stderr))
            os.replace(obj + ".tmp", obj)
            if verbose or ptxas_info:
                sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(units), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, units))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(" ".join(extra))
    return LIB


HARNESS_SRC = os.path.join(HERE, "harness", "nlse_harness.c")
HARNESS = os.path.join(HERE, "harness", "nlse_harness")


def build_harness(force: bool = False) -> str:
    """Compile the standalone C harness (nlsemagic_gb300/harness/nlse_harness)
    against the library's C ABI with the host C compiler; it finds the
    library next to itself at run time (rpath $ORIGIN/..)."""
    lib = build()
    if force or _stale(HARNESS, [HARNESS_SRC, lib, os.path.join(INCLUDE, "nlse_gb300.h")]):
        cc = os.environ.get("CC", "gcc")
        tmp = HARNESS + ".tmp%d" % os.getpid()
        cmd = [cc, "-std=gnu11", "-O2", "-Wall", "-Wextra", "-ffp-contract=off", "-I", INCLUDE,
               HARNESS_SRC, "-o", tmp, "-L", HERE, "-lnlse_gb300", "-Wl,-rpath,$ORIGIN/..",
               "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("harness build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, HARNESS)
    return HARNESS


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                ptxas_info="--ptxas" in sys.argv))
