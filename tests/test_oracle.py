"""Pin the C oracle (oracle/nlse_oracle.c) before it is trusted as the checker.

1. Bit-for-bit against the committed golden vectors made by the reference's
   own C integrators (tests/golden/make_golden.py) -- runs everywhere.
2. Bit-for-bit against the live reference build (oracle/_ref) on fresh
   random cases -- only where the reference checkout exists.
3. Known-answer checks from the reference's research scripts: order of
   accuracy (CD 2, 2SHOC 4; src/NLSEmagic1D/NLSEmagic1D_FRS.m:693), mass
   conservation (:583-586) and the grey-soliton closed form (:542).
"""
import itertools
import math
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_vectors.npz")


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64)
    b = np.ascontiguousarray(b, dtype=np.complex128).view(np.float64)
    return np.array_equal(a, b, equal_nan=True)


def golden_cases():
    z = np.load(GOLDEN)
    for n in range(int(z["ncases"])):
        pre = "c%03d_" % n
        ndim, method, prec, BC, chunk = (int(x) for x in z[pre + "meta"])
        s, a, h2, k = (float(x) for x in z[pre + "par"])
        yield n, dict(U=z[pre + "U"], V=z[pre + "V"], out=z[pre + "out"], ndim=ndim,
                      method=method, precision=prec, BC=BC, chunk=chunk, s=s, a=a, h2=h2, k=k)


def test_golden_file_present():
    assert os.path.exists(GOLDEN)
    z = np.load(GOLDEN)
    assert int(z["ncases"]) >= 70


@pytest.mark.parametrize("n,case", list(golden_cases()), ids=lambda v: str(v) if isinstance(v, int) else "")
def test_oracle_matches_golden(n, case):
    c = case
    # Reference CPU semantics: no MSD guard; the single-precision quirk on.
    flags = oracle.REF_QUIRKS if c["precision"] == 1 else 0
    got = oracle.take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"], c["chunk"], c["k"],
                            method=c["method"], precision=c["precision"], flags=flags)
    assert got.shape == c["out"].shape
    assert bits_equal(got, c["out"]), "case %d differs from the reference output" % n


def test_msd_guard_only_changes_nan_points():
    z = np.load(GOLDEN)
    # the golden MSD zero-neighbour case: reference result contains NaN
    for n, c in golden_cases():
        if c["ndim"] == 3 and c["BC"] == 2 and np.count_nonzero(c["U"] == 0) == 1:
            assert np.isnan(c["out"]).any()
            guarded = oracle.take_steps(c["U"], c["V"], c["s"], c["a"], c["h2"], c["BC"],
                                        c["chunk"], c["k"], method=c["method"],
                                        precision=c["precision"], flags=oracle.MSD_GUARD)
            assert np.isfinite(guarded).all()
            ok = np.isfinite(c["out"])
            assert bits_equal(guarded[ok], c["out"][ok])
            break
    else:
        pytest.fail("zero-neighbour golden case missing")
    del z


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("ndim,method,prec,BC",
                         [c for c in itertools.product([1, 2, 3], [1, 2], [2, 1], [1, 2, 3, 4])
                          if not (c[3] == 4 and c[0] != 1)])
def test_oracle_matches_live_reference(ndim, method, prec, BC):
    if ndim == 2 and method == 2 and prec == 1 and BC in (1, 2):
        pytest.skip("reference reads an uninitialised 1/a here (NLSE2D_TAKE_STEPS_2SHOC_F.c:299)")
    rng = np.random.default_rng(1234 + 100 * ndim + 10 * method + BC + prec)
    shape = {1: (23,), 2: (9, 8), 3: (6, 5, 7)}[ndim]
    U = (0.8 + 0.3 * rng.standard_normal(shape)) + 0.3j * rng.standard_normal(shape)
    V = 0.2 * rng.random(shape)
    args = (U, V, 1.0, 0.7, 0.12, BC, 6, 0.003)
    ref = oracle.ref_take_steps(*args, method=method, precision=prec)
    got = oracle.take_steps(*args, method=method, precision=prec,
                            flags=oracle.REF_QUIRKS if prec == 1 else 0)
    assert bits_equal(got, ref)


@pytest.mark.parametrize("ndim,method,prec", list(itertools.product([1, 2, 3], [1, 2], [2, 1])))
def test_oracle_thread_count_does_not_change_bits(ndim, method, prec):
    # The large parity runs spread one solve over threads; each grid sweep
    # writes every point from values no other point of that sweep writes.
    shape = {1: (301,), 2: (41, 37), 3: (19, 17, 23)}[ndim]
    rng = np.random.default_rng(31 + 10 * ndim + method + prec)
    U = (1 + 0.2 * rng.standard_normal(shape)) + 0.2j * rng.standard_normal(shape)
    V = 0.1 * rng.random(shape)
    for BC in (1, 2, 3):
        args = (U, V, -1.0, 1.0, 0.1, BC, 4, 0.002)
        try:
            oracle.set_threads(1)
            one = oracle.take_steps(*args, method=method, precision=prec)
            oracle.set_threads(4)
            many = oracle.take_steps(*args, method=method, precision=prec)
        finally:
            oracle.set_threads(1)
        assert bits_equal(one, many), BC


def test_oracle_rejects_bad_arguments():
    U = np.ones(8, dtype=complex)
    with pytest.raises(ValueError):
        oracle.take_steps(U[:2], np.zeros(2), -1, 1, 0.01, 2, 1, 1e-3)
    with pytest.raises(ValueError):
        oracle.take_steps(np.ones((3, 3)), np.zeros((3, 3)), -1, 1, 0.01, 4, 1, 1e-3)
    with pytest.raises(ValueError):
        oracle.take_steps(U, np.zeros(8), -1, 1, 0.01, 2, 1, 1e-3, method=3)


# ---- known-answer checks (the reference's own validation strategy) --------

def _linear_gaussian_error(method, h, T=0.5, L=12.0):
    # s = 0, V = x^2, a = 1: U = exp(-x^2/2) exp(-i t) is an eigenstate
    # (src/NLSEmagic1D/NLSEmagic1D_FRS.m:538 with a = 1).  k small enough
    # that the time error is negligible; Dirichlet boundary far away.
    n = int(round(2 * L / h)) + 1
    x = -L + h * np.arange(n)
    U0 = np.exp(-x * x / 2).astype(complex)
    V = x * x
    k = 0.05 * h * h
    steps = int(round(T / k))
    out = oracle.take_steps(U0, V, 0.0, 1.0, h * h, 1, steps, k, method=method)
    exact = np.exp(-x * x / 2) * np.exp(-1j * steps * k)
    return np.sqrt(np.mean(np.abs(out - exact) ** 2))


@pytest.mark.parametrize("method,order", [(1, 2.0), (2, 4.0)])
def test_order_of_accuracy(method, order):
    e1 = _linear_gaussian_error(method, 0.4)
    e2 = _linear_gaussian_error(method, 0.2)
    m = math.log(e1 / e2) / math.log(2.0)
    assert abs(m - order) < 0.35, "observed order %.3f" % m


def test_mass_conserved_and_grey_soliton_tracks_closed_form():
    from nlsemagic_gb300 import workloads as W
    w = W.grey_soliton_1d(N=1024, noise=0.0)
    U = w.U
    m0 = W.mass(U, w.h, 1)
    steps = 200
    out = oracle.take_steps(U, w.V, w.s, w.a, w.h2, w.BC, steps, w.k, method=w.method)
    # mass drift small
    assert abs(W.mass(out, w.h, 1) - m0) / m0 < 1e-6
    # exact grey soliton moving at speed c: U(x, t) = U0(x - c t) e^{-i t}
    # (s = -1, background 1), cf. src/NLSEmagic1D/NLSEmagic1D_FRS.m:542
    c = w.meta["c"]
    t = steps * w.k
    x = -51.2 + w.h * np.arange(1024)
    wv = math.sqrt(1 - c * c / 2)
    exact = (1j * c / math.sqrt(2) + wv * np.tanh(wv * (x - c * t) / math.sqrt(2))) * np.exp(-1j * t)
    inner = slice(200, 824)
    err = np.max(np.abs(out[inner] - exact[inner]))
    assert err < 5e-3, err


# ---- 3D vorticity (src/NLSEmagic3D/rmc_vorticity3D.c) --------------------------
VORT_SHAPES = [(5, 6, 7), (9, 8, 10), (3, 3, 3), (12, 5, 4), (40, 33, 21)]


@pytest.mark.parametrize("shape", VORT_SHAPES)
def test_vorticity_oracle_matches_reference(shape):
    if not oracle.ref_available():
        pytest.skip("reference checkout not present")
    rng = np.random.default_rng(sum(shape))
    U = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    U[1, 1, 1] = 0.0  # veps keeps |U| = 0 finite
    lh2, veps = 1.0 / (2 * 0.3), 1e-6
    got = oracle.vorticity3d(U, lh2, veps)
    want = oracle.ref_vorticity3d(U, lh2, veps)
    M, N, L = shape
    interior = np.zeros(shape, bool)
    interior[1:M - 1, 1:N - 1, 1:L - 1] = True
    for g, w in zip(got, want):
        # interior points never read the reference's uninitialised edge
        # gradients: bit-identical
        assert np.array_equal(g[interior], w[interior])
        # the edges and corners are 0 in both
        edge = np.zeros(shape, bool)
        for a in range(3):
            for b in range(a + 1, 3):
                sl = [slice(None)] * 3
                for ia in (0, shape[a] - 1):
                    for ib in (0, shape[b] - 1):
                        sl[a], sl[b] = ia, ib
                        edge[tuple(sl)] = True
        assert np.all(g[edge] == 0) and np.all(w[edge] == 0)
    if U.size >= 16384:
        # large enough that the reference's scratch comes from freshly mapped
        # (zeroed) memory: its edge gradients are 0 as here, every point agrees
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_vorticity_of_a_straight_vortex_line():
    # U = (x + i y)/r-like charge-1 line along the slowest axis: the vorticity
    # points along that axis and its magnitude integrates to ~2 pi / |v| scale
    h = 0.25
    n = 24
    ax = (np.arange(n) - (n - 1) / 2) * h
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")  # fastest first: (k, j, i)
    # in the routine's axes: x = slowest (i), y = middle (j), z = fastest (k);
    # a line along x winds in the (y, z) plane
    U = np.tanh(np.hypot(Y, Z)) * np.exp(1j * np.arctan2(Y, Z))
    wx, wy, wz, W = oracle.vorticity3d(U, 1 / (2 * h), 1e-12)
    core = W[n // 2 - 2:n // 2 + 2, n // 2 - 2:n // 2 + 2, n // 2]
    far = W[2, 2, n // 2]
    assert core.max() > 10 * far
    mid = (slice(3, n - 3),) * 3
    assert np.abs(wx[mid]).max() > 5 * max(np.abs(wy[mid]).max(), np.abs(wz[mid]).max())


# ---- 2D cubic-quintic 2SHOC (src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c) -----
@pytest.mark.parametrize("shape", [(9, 7), (16, 23), (5, 5), (40, 31)])
@pytest.mark.parametrize("BC", [1, 2, 3])
def test_cq2d_oracle_matches_reference(shape, BC):
    if not oracle.ref_available():
        pytest.skip("reference checkout not present")
    rng = np.random.default_rng(shape[0] * 7 + BC)
    U = (1 + 0.3 * rng.standard_normal(shape)) + 0.3j * rng.standard_normal(shape)
    V = 0.1 * rng.random(shape)
    args = (U, V, -1.0, 0.3, 1.2, 0.09, BC, 7, 0.004)
    got = oracle.cq2d(*args, flags=0)  # the file has no zero-neighbour guard
    want = oracle.ref_cq2d(*args)
    assert np.array_equal(np.ascontiguousarray(got).view(np.float64),
                          np.ascontiguousarray(want).view(np.float64))


def test_cq2d_reduces_to_cubic_interior_when_s2_is_zero():
    # with s2 = 0 and Dirichlet / Laplacian-zero boundaries the cubic-quintic
    # file's formulas are those of the cubic 2D 2SHOC integrator up to
    # operand order: the two agree to rounding
    rng = np.random.default_rng(11)
    U = (1 + 0.2 * rng.standard_normal((20, 18))) + 0.2j * rng.standard_normal((20, 18))
    V = 0.05 * rng.random((20, 18))
    for BC in (1, 3):
        a = oracle.cq2d(U, V, -1.0, 0.0, 1.0, 0.09, BC, 5, 0.004)
        b = oracle.take_steps(U, V, -1.0, 1.0, 0.09, BC, 5, 0.004, method=2, precision=2)
        assert np.max(np.abs(a - b)) < 1e-12
