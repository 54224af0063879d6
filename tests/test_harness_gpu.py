"""The standalone C harness (nlsemagic_gb300/harness/nlse_harness.c).

The harness is a C program with no Python and no MATLAB in it: it makes the
seeded initial data of configurations 1-3 itself (splitmix64 + Box-Muller),
advances them chunk by chunk through the library's C ABI (the one-shot v2
functions, or the resident solver) and prints one JSON line per run.  Here it
runs on reduced grids and its dumped inputs and results are checked against
the C oracle: FP64 and FP32 bit for bit, the mixed class within 1e-6
relative L2 of the FP64 oracle.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def run_harness(tmp, *args):
    from nlsemagic_gb300 import build as B
    exe = B.build_harness()
    r = subprocess.run([exe, "--dump", str(tmp)] + list(args), capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    return [json.loads(ln) for ln in r.stdout.splitlines() if ln.strip()]


def shape_of(line):
    return tuple(line["grid"][:line["ndim"]])


def planes(path, shape, count):
    n = int(np.prod(shape))
    a = np.fromfile(path, dtype="<f8")
    assert a.size == count * n
    return [a[i * n:(i + 1) * n].reshape(shape, order="F") for i in range(count)]


@pytest.mark.parametrize("mode", ["oneshot", "resident"])
def test_harness_matches_oracle(gpu_lib, tmp_path, mode):
    # 48: a grid where the config-3 rings stay clear of the MSD faces (at 40 and
    # 64 points a ring core next to a face drives the FP64 oracle itself to NaN)
    lines = run_harness(tmp_path, "--config", "1,2,3", "--n", "48", "--steps", "36",
                        "--chunk", "12", "--mode", mode)
    assert len(lines) == 9
    for ln in lines:
        assert "error" not in ln, ln
        assert ln["mode"] == mode and ln["chunks"] == 3 and ln["steps"] == 36
        c = ln["config"]
        shape = shape_of(ln)
        ur, ui, V = planes(tmp_path / ("c%d_in.bin" % c), shape, 3)
        U = ur + 1j * ui
        method = 1 if ln["method"] == "CD" else 2
        h2 = ln["h"] * ln["h"]
        got_r, got_i = planes(tmp_path / ("c%d_%s_%s.bin" % (c, ln["precision"], mode)), shape, 2)
        got = got_r + 1j * got_i
        args = (U, V, -1.0, 1.0, h2, ln["bc"], 36, ln["k"])
        if ln["precision"] == "fp64":
            ref = oracle.take_steps(*args, method=method, precision=2, flags=oracle.MSD_GUARD)
            assert bits_equal(got, ref), ln
        elif ln["precision"] == "fp32":
            ref = oracle.take_steps(*args, method=method, precision=1, flags=oracle.MSD_GUARD)
            assert bits_equal(got, ref), ln
        else:
            ref = oracle.take_steps(*args, method=method, precision=2, flags=oracle.MSD_GUARD)
            err = float(np.linalg.norm((got - ref).ravel()) / np.linalg.norm(ref.ravel()))
            assert err <= MIXED_TOL, (ln, err)
            assert ln["rel_l2_vs_fp64"] <= MIXED_TOL
        mass0 = float(np.sum(np.abs(U) ** 2)) * ln["h"] ** ln["ndim"]
        assert ln["mass0"] == pytest.approx(mass0, rel=1e-12)


def test_harness_default_configurations(gpu_lib, tmp_path):
    # configuration 1 at its own size and length (1024 points, 1000 steps in
    # chunks of 100), through the one-shot FP64 call
    lines = run_harness(tmp_path, "--config", "1", "--precision", "fp64")
    (ln,) = lines
    assert ln["grid"] == [1024, 1, 1] and ln["steps"] == 1000 and ln["chunks"] == 10
    assert ln["method"] == "CD" and ln["bc"] == 2 and ln["k"] == 0.005
    ur, ui, V = planes(tmp_path / "c1_in.bin", (1024,), 3)
    ref = oracle.take_steps(ur + 1j * ui, V, -1.0, 1.0, ln["h"] ** 2, 2, 1000, 0.005, method=1,
                            precision=2, flags=oracle.MSD_GUARD)
    got_r, got_i = planes(tmp_path / "c1_fp64_oneshot.bin", (1024,), 2)
    assert bits_equal(got_r + 1j * got_i, ref)
    # the MSD boundary lets mass drift a little (the oracle shows 2.5e-5 on this
    # workload); a blow-up would show orders of magnitude more
    assert ln["mass_rel_drift"] < 1e-3
