"""Generate golden input/output vectors from the reference's own C integrators.

Run in a checkout where the reference sources exist (``oracle/build.py``
compiles them unmodified against ``oracle/mexshim``):

    python tests/golden/make_golden.py

Writes ``tests/golden/ref_vectors.npz``.  Each case stores the seeded inputs,
the call arguments and the reference output of ``U = NAME(U, V, s, a, h2, BC,
chunk_size, k)``.  The vectors pin the project's C oracle (and, through it, the
GPU library) to the reference on machines where the reference is absent.

Cases: every (dimension, method, precision, BC) combination the reference
files implement, on a generic and a minimal grid, plus a real-valued input,
an MSD case whose interior neighbour is exactly zero (the reference yields
NaN there; kept as evidence of the zero-division), and a short run of the
1D grey-soliton workload.
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

OUT = os.path.join(HERE, "ref_vectors.npz")

SHAPES = {1: [(19,), (4,)], 2: [(7, 9), (3, 4)], 3: [(5, 6, 7), (3, 4, 3)]}


def cases():
    rng = np.random.default_rng(20261203)
    out = []
    for ndim, method, prec, BC in itertools.product([1, 2, 3], [1, 2], [2, 1], [1, 2, 3, 4]):
        if BC == 4 and ndim != 1:
            continue
        for shp in SHAPES[ndim]:
            if BC == 4 and shp[-1] < 4:
                continue
            # the single-precision 2D 2SHOC file reads an uninitialised 1/a for BC 1, 2
            if ndim == 2 and method == 2 and prec == 1 and BC in (1, 2):
                continue
            U = (1 + 0.3 * rng.standard_normal(shp)) + 1j * (0.3 * rng.standard_normal(shp))
            V = 0.1 * rng.random(shp)
            s = float(rng.choice([-1.0, 1.0]))
            a = float(rng.uniform(0.5, 2.0))
            h2 = float(rng.uniform(0.05, 0.2))
            k = 0.05 * h2 / a
            chunk = int(rng.integers(3, 9))
            out.append(dict(ndim=ndim, method=method, precision=prec, BC=BC, U=U, V=V, s=s, a=a,
                            h2=h2, chunk=chunk, k=k))
    # real-valued input (the reference zero-fills the imaginary plane)
    U = 1 + 0.2 * rng.standard_normal((6, 8))
    out.append(dict(ndim=2, method=1, precision=2, BC=2, U=U.astype(np.float64),
                    V=np.zeros((6, 8)), s=-1.0, a=1.0, h2=0.1, chunk=5, k=0.002))
    # MSD with an exactly-zero interior neighbour: reference output is NaN
    U = np.ones((5, 5, 5), dtype=np.complex128)
    U[1, 1, 1] = 0
    out.append(dict(ndim=3, method=1, precision=2, BC=2, U=U, V=np.zeros((5, 5, 5)), s=-1.0,
                    a=1.0, h2=0.09, chunk=1, k=0.001))
    # 1D grey soliton, N=256 on [-12.8, 12.8), MSD, 40 steps
    x = -12.8 + 0.1 * np.arange(256)
    c = 0.5
    w = np.sqrt(1 - c * c / 2)
    U = 1j * c / np.sqrt(2) + w * np.tanh(w * x / np.sqrt(2))
    out.append(dict(ndim=1, method=1, precision=2, BC=2, U=U, V=np.zeros(256), s=-1.0, a=1.0,
                    h2=0.01, chunk=40, k=0.005))
    return out


def main():
    if not oracle.ref_available():
        raise SystemExit("reference sources not found; cannot regenerate golden vectors")
    arrays = {}
    cs = cases()
    for n, c in enumerate(cs):
        out = oracle.ref_take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], c["chunk"],
                                    c["k"], method=c["method"], precision=c["precision"])
        pre = "c%03d_" % n
        arrays[pre + "U"] = np.asarray(c["U"])
        arrays[pre + "V"] = c["V"]
        arrays[pre + "out"] = out
        arrays[pre + "meta"] = np.array([c["ndim"], c["method"], c["precision"], c["BC"],
                                         c["chunk"]], dtype=np.int64)
        arrays[pre + "par"] = np.array([c["s"], c["a"], c["h2"], c["k"]], dtype=np.float64)
    arrays["ncases"] = np.array(len(cs))
    np.savez_compressed(OUT, **arrays)
    print("wrote %d cases to %s (%d bytes)" % (len(cs), OUT, os.path.getsize(OUT)))


if __name__ == "__main__":
    main()
