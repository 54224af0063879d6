"""Seeded synthetic workloads: the initial data, potentials and parameters of
the benchmark configurations.

Grids are cell-vertex, x_i = x_min + i h, identical on every axis; arrays are
MATLAB-shaped (first index fastest).  All randomness comes from
``numpy.random.default_rng(seed)`` (PCG64), so every machine generates the
same inputs for the same seed.

* :func:`grey_soliton_1d` -- 1D CD, N = 1024 on [-51.2, 51.2), MSD, co-moving
  dark (grey) soliton with c = 0.5 plus 1e-4 complex Gaussian noise; the
  reference's grey-soliton initial condition (src/NLSEmagic1D/NLSEmagic1D_FRS.m:219-224).
* :func:`dark_vortices_2d` -- 2D 2SHOC, 512^2 on [-64, 64)^2, Dirichlet,
  product of four charge +-1 vortices tanh(r_j) e^{+-i theta_j} at seeded
  centres, times exp(i 1e-3 g) (the "Gaussian phase noise" read as a phase).
* :func:`vortex_rings_3d` -- 3D, 320^3 on [-48, 48)^3, MSD, harmonic trap
  V = 0.5 w^2 r^2 (w = 0.02), Thomas-Fermi background sqrt(max(0, 1 - V))
  times four vortex rings (radius 6-10, seeded centres and orientations,
  core profile tanh(d) e^{i phi}).
* :func:`batch_instances` -- the uneven batch of 1D/2D solves.
* :func:`serving_requests` -- the Poisson request stream of the serving loop.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    U: np.ndarray
    V: np.ndarray
    s: float
    a: float
    h: float
    BC: int
    method: int
    k: float
    steps: int
    chunk: int
    meta: dict = field(default_factory=dict)

    @property
    def h2(self):
        return self.h * self.h

    @property
    def ndim(self):
        return self.U.ndim if min(self.U.shape) > 1 else 1

    @property
    def points(self):
        return int(self.U.size)


def linear_stability_k(ndim, method, h, a):
    """h^2 / (ndim sqrt(2) a) for CD, 3/4 of that for 2SHOC
    (src/NLSEmagic3D/NLSEmagic3D.m:154-163)."""
    klin = h * h / (ndim * math.sqrt(2.0) * a)
    return klin * 0.75 if method == 2 else klin


def axis(n, xmin, h):
    return xmin + h * np.arange(n, dtype=np.float64)


def grey_soliton_1d(seed=1000, N=1024, h=0.1, c=0.5, noise=1e-4, steps=1000, chunk=100):
    x = axis(N, -N * h / 2, h)
    w = math.sqrt(1 - c * c / 2)
    U = 1j * c / math.sqrt(2) + w * np.tanh(w * x / math.sqrt(2))
    rng = np.random.default_rng(seed)
    U = U + noise * (rng.standard_normal(N) + 1j * rng.standard_normal(N))
    return Workload("1d_cd_grey_soliton_N%d" % N, U.astype(np.complex128), np.zeros(N), s=-1.0,
                    a=1.0, h=h, BC=2, method=1, k=0.005, steps=steps, chunk=chunk,
                    meta=dict(c=c, seed=seed))


def dark_vortices_2d(seed=1001, n=512, h=0.25, nvort=4, steps=2000, method=2, phase_noise=1e-3,
                     span=20.0):
    x = axis(n, -n * h / 2, h)
    X, Y = np.meshgrid(x, x, indexing="ij")
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-span, span, size=(nvort, 2))
    charges = np.array([1, -1] * ((nvort + 1) // 2))[:nvort]
    rng.shuffle(charges)
    U = np.ones((n, n), dtype=np.complex128)
    for (cx, cy), q in zip(centres, charges):
        dx, dy = X - cx, Y - cy
        r = np.hypot(dx, dy)
        U *= np.tanh(r) * np.exp(1j * q * np.arctan2(dy, dx))
    U *= np.exp(1j * phase_noise * rng.standard_normal((n, n)))
    k = 0.8 * linear_stability_k(2, method, h, 1.0)
    return Workload("2d_%s_dark_vortices_%dx%d" % ("2shoc" if method == 2 else "cd", n, n), U,
                    np.zeros((n, n)), s=-1.0, a=1.0, h=h, BC=1, method=method, k=k, steps=steps,
                    chunk=steps, meta=dict(seed=seed, centres=centres.tolist(),
                                           charges=charges.tolist()))


def _unit_vectors(rng, m):
    v = rng.standard_normal((m, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def vortex_rings_3d(seed=1002, n=320, h=0.3, omega=0.02, nrings=4, steps=500, method=2,
                    dtype=np.complex128):
    x = axis(n, -n * h / 2, h)
    rng = np.random.default_rng(seed)
    radii = rng.uniform(6.0, 10.0, size=nrings)
    centres = rng.uniform(-15.0, 15.0, size=(nrings, 3))
    normals = _unit_vectors(rng, nrings)
    X = x[:, None, None]
    Y = x[None, :, None]
    Z = x[None, None, :]
    V = 0.5 * omega * omega * (X * X + Y * Y + Z * Z)
    V = np.broadcast_to(V, (n, n, n)).astype(np.float64)
    U = np.sqrt(np.maximum(0.0, 1.0 - V)).astype(dtype)
    for R, c, nv in zip(radii, centres, normals):
        dx = X - c[0]
        dy = Y - c[1]
        dz = Z - c[2]
        zax = dx * nv[0] + dy * nv[1] + dz * nv[2]            # axial coordinate
        rho = np.sqrt(np.maximum(dx * dx + dy * dy + dz * dz - zax * zax, 0.0))
        dr = rho - R
        d = np.sqrt(dr * dr + zax * zax)                        # distance to the core circle
        U *= np.tanh(d) * np.exp(1j * np.arctan2(zax, dr))
        del dx, dy, dz, zax, rho, dr, d
    k = 0.8 * linear_stability_k(3, method, h, 1.0)
    return Workload("3d_%s_vortex_rings_%d^3" % ("2shoc" if method == 2 else "cd", n), U, V,
                    s=-1.0, a=1.0, h=h, BC=2, method=method, k=k, steps=steps, chunk=steps,
                    meta=dict(seed=seed, omega=omega, radii=radii.tolist(),
                              centres=centres.tolist(), normals=normals.tolist()))


def sech_or_tanh(x, s):
    """Bright soliton sech(x) for s = +1, dark soliton tanh(x) for s = -1."""
    if s > 0:
        with np.errstate(over="ignore"):  # cosh overflows far out: sech -> 0 there
            return 1.0 / np.cosh(x)
    return np.tanh(x)


@dataclass
class Instance:
    ndim: int
    shape: tuple
    U: np.ndarray
    V: np.ndarray
    s: float
    a: float
    h: float
    BC: int
    method: int
    k: float
    steps: int
    precision: int


def _instance(rng, ndim, n, steps, precision, omega_scale=1.0):
    a = float(rng.uniform(0.5, 2.0))
    s = float(rng.choice([-1.0, 1.0]))
    method = int(rng.integers(1, 3))
    h = 0.1 if ndim == 1 else 0.25
    L = n * h
    x = axis(n, -L / 2, h)
    omega = omega_scale * 4.0 / L
    if ndim == 1:
        V = 0.5 * omega * omega * x * x
        U = sech_or_tanh(x / math.sqrt(2 * a), s).astype(np.complex128)
        shape = (n,)
    elif ndim == 2:
        X, Y = np.meshgrid(x, x, indexing="ij")
        V = 0.5 * omega * omega * (X * X + Y * Y)
        r = np.hypot(X, Y)
        U = (sech_or_tanh(r / math.sqrt(2 * a), s) * np.exp(1j * np.arctan2(Y, X))).astype(
            np.complex128)
        if s > 0:
            U = (1.0 / np.cosh(r / math.sqrt(2 * a))).astype(np.complex128)
        shape = (n, n)
    else:
        X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
        V = 0.5 * omega * omega * (X * X + Y * Y + Z * Z)
        r = np.sqrt(X * X + Y * Y + Z * Z)
        U = sech_or_tanh(r / math.sqrt(2 * a), s).astype(np.complex128)
        shape = (n, n, n)
    k = 0.8 * linear_stability_k(ndim, method, h, a)
    return Instance(ndim, shape, U, np.asarray(V, dtype=np.float64), s, a, h,
                    BC=1 if s > 0 else 2, method=method, k=k, steps=steps, precision=precision)


def batch_instances(seed=1003, count=512, steps=1000, frac_1d=0.6, n1=(256, 16384),
                    n2=(64, 512), precision=3):
    """Uneven batch: 60% 1D (N log-uniform in [256, 16384]) and 40% 2D (side
    log-uniform in [64, 512]); per solve seeded a in [0.5, 2], s = +-1, a
    harmonic trap, CD or 2SHOC 50/50, sech (s = +1) or tanh (s = -1) data."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        if rng.random() < frac_1d:
            n = int(round(math.exp(rng.uniform(math.log(n1[0]), math.log(n1[1])))))
            out.append(_instance(rng, 1, n, steps, precision))
        else:
            n = int(round(math.exp(rng.uniform(math.log(n2[0]), math.log(n2[1])))))
            out.append(_instance(rng, 2, n, steps, precision))
    return out


@dataclass
class Request:
    rid: int
    arrival: float
    inst: Instance


def serving_requests(seed=1004, count=20000, rate=200.0, ratio=(5, 4, 1),
                     n1=(512, 65536), n2=(64, 1024), n3=(32, 256), steps=(100, 5000),
                     materialize=True):
    """Poisson arrivals (mean rate `rate` per second); dims 1D:2D:3D = 5:4:1;
    sizes and step counts log-uniform; precision class FP64 or mixed 50/50."""
    rng = np.random.default_rng(seed)
    t = 0.0
    p = np.array(ratio, dtype=float) / sum(ratio)
    out = []
    for rid in range(count):
        t += rng.exponential(1.0 / rate)
        ndim = int(rng.choice([1, 2, 3], p=p))
        lo, hi = {1: n1, 2: n2, 3: n3}[ndim]
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        nsteps = int(round(math.exp(rng.uniform(math.log(steps[0]), math.log(steps[1])))))
        prec = 2 if rng.random() < 0.5 else 3
        inst = _instance(rng, ndim, n, nsteps, prec) if materialize else (ndim, n, nsteps, prec)
        out.append(Request(rid, t, inst))
    return out


def rel_l2(a, b):
    """||a - b|| / ||b|| over all points."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def mass(U, h, ndim):
    """sum |U|^2 h^ndim."""
    return float(np.sum(np.abs(U) ** 2) * h ** ndim)
