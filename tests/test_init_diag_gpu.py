"""Initial conditions generated on the device and per-chunk diagnostics:
the generators against the numpy formulas of the workloads (to a few ulps:
transcendental functions differ in the last bits between libraries), the
seeded noise's statistics and reproducibility, the diagnostics against
numpy reductions of the downloaded state, and the closed-form 1D errors."""
import math

import numpy as np
import pytest

from nlsemagic_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def solver(shape, prec, method=2, BC=1, s=-1.0, a=1.0, h=0.3, k=1e-3):
    import nlsemagic_gb300 as ng
    return ng.Solver(shape, method=method, precision=prec, BC=BC, s=s, a=a, h2=h * h, k=k)


def test_grey_soliton_matches_workload(gpu_lib):
    import nlsemagic_gb300 as ng
    w = W.grey_soliton_1d(noise=0.0)
    with solver(w.U.shape, ng.PREC_DOUBLE, BC=2, h=w.h) as sv:
        sv.init_ic(ng.IC_GREY, om=-1.0, c=0.5, x0=0.0)
        assert rel_max(sv.download(), w.U) < 1e-13


@pytest.mark.parametrize("kind", ["sech", "tanh", "gauss"])
def test_1d_solitons(gpu_lib, kind):
    import nlsemagic_gb300 as ng
    n, h, a, om, c, x0 = 400, 0.1, 1.3, 0.8, 0.4, 2.0
    s = 1.0 if kind == "sech" else -1.0
    x = -n * h / 2 + h * np.arange(n)
    if kind == "sech":
        want = math.sqrt(2 * om / s) / np.cosh(math.sqrt(om / a) * (x - x0)) * np.exp(
            1j * c / (2 * a) * x)
        k_ = ng.IC_SECH
    elif kind == "tanh":
        om = -om
        want = math.sqrt(om / s) * np.tanh(math.sqrt(abs(om / (2 * a))) * (x - x0)) * np.exp(
            1j * c / (2 * a) * x)
        k_ = ng.IC_TANH
    else:
        want = np.exp(-x * x / (2 * a)).astype(complex)
        k_ = ng.IC_GAUSS
    with solver((n,), ng.PREC_DOUBLE, s=s, a=a, h=h) as sv:
        sv.init_ic(k_, om=om, c=c, x0=x0)
        assert rel_max(sv.download(), want) < 1e-13
        # at t = 0 the closed form is the initial condition itself
        assert max(sv.error_1d(k_, 0.0, om=om, c=c, x0=x0)) < 1e-13


def test_vortices_and_rings_match_workloads(gpu_lib):
    import nlsemagic_gb300 as ng
    w2 = W.dark_vortices_2d(n=96, phase_noise=0.0, span=8.0)
    items = [(cx, cy, q) for (cx, cy), q in zip(w2.meta["centres"], w2.meta["charges"])]
    with solver(w2.U.shape, ng.PREC_DOUBLE, h=w2.h) as sv:
        sv.init_ic(ng.IC_VORTICES, items=items)
        assert rel_max(sv.download(), w2.U) < 1e-12
    w3 = W.vortex_rings_3d(n=40, h=0.6)
    rings = [tuple(c) + tuple(nv) + (R,) for c, nv, R in
             zip(w3.meta["centres"], w3.meta["normals"], w3.meta["radii"])]
    with solver(w3.U.shape, ng.PREC_DOUBLE, BC=2, h=w3.h) as sv:
        sv.init_ic(ng.IC_RINGS, items=rings, omega=w3.meta["omega"])
        assert rel_max(sv.download(), w3.U) < 1e-12


def test_seeded_noise(gpu_lib):
    import nlsemagic_gb300 as ng
    n = 20000
    out = []
    for seed in (7, 7, 8):
        with solver((n,), ng.PREC_DOUBLE, s=1.0) as sv:
            sv.init_ic(ng.IC_GAUSS, noise_kind=ng.NOISE_ADD, noise=0.01, seed=seed)
            out.append(sv.download())
    assert np.array_equal(out[0], out[1])
    assert not np.array_equal(out[0], out[2])
    x = -n * 0.3 / 2 + 0.3 * np.arange(n)
    g = (out[0] - np.exp(-x * x / 2)) / 0.01
    for comp in (g.real, g.imag):
        assert abs(comp.mean()) < 0.05 and abs(comp.std() - 1) < 0.05


@pytest.mark.parametrize("prec", [1, 2, 3])
def test_diagnostics_match_numpy(gpu_lib, prec):
    import nlsemagic_gb300 as ng
    rng = np.random.default_rng(prec)
    U = rng.standard_normal((30, 20)) + 1j * rng.standard_normal((30, 20))
    U[3, 4] = np.nan
    U[7, 1] = complex(np.inf, 0)
    h = 0.3
    with solver(U.shape, prec, h=h) as sv:
        sv.upload(U, np.zeros(U.shape))
        d = sv.diagnostics()
        got = sv.download()
    fin = np.isfinite(got.real) & np.isfinite(got.imag)
    assert d["nonfinite"] == int((~fin).sum()) == 2
    q = np.abs(got[fin]) ** 2
    assert abs(d["mass"] - q.sum() * h * h) <= 1e-12 * q.sum() * h * h
    assert abs(d["max_abs2"] - q.max()) <= 1e-15 * q.max()
    assert d["max_re"] == got.real[fin].max()


def test_bright_soliton_error_is_second_order_small(gpu_lib):
    # the sech soliton is an exact solution: after t = 1 the CD scheme's
    # error against the closed form shrinks ~4x when h halves
    import nlsemagic_gb300 as ng
    errs = []
    for h in (0.2, 0.1):
        n = int(round(40 / h))
        k = 0.5 * ng.linear_stability_k(1, 1, h, 1.0)
        steps = int(round(1.0 / k))
        with ng.Solver((n,), method=1, precision=ng.PREC_DOUBLE, BC=1, s=1.0, a=1.0, h2=h * h,
                       k=k) as sv:
            sv.init_ic(ng.IC_SECH, om=1.0, c=0.5, x0=-5.0)
            sv.run(steps)
            errs.append(max(sv.error_1d(ng.IC_SECH, steps * k, om=1.0, c=0.5, x0=-5.0)))
    assert errs[1] < errs[0] / 3
