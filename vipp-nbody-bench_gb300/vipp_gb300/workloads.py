"""Seeded synthetic initial conditions of the benchmark workloads (host, numpy).

The reference draws its one initial condition on the host
(Problem::initialize, gravity/include/problem.hpp:188-211); the GPU generator
of that model is ``Solver.init_plummer``. These are the larger synthetic
workloads the solver is measured on, as (x, v) AoS float64 arrays in
G = 1 units:

  plummer    a Plummer sphere (total mass 1, scale radius 1) with the
             inverse-CDF radius capped at r_max and speeds by von Neumann
             rejection from the Plummer distribution function;
  uniform    particles uniform in the unit cube [0, 1)^3 at rest;
  clustered  the adaptive-depth stress workload: 8 equal-mass Plummer
             clusters (scale radii uniform in [0.01, 0.1], centres uniform in
             [0, 1)^3, bulk velocities Gaussian with sigma 0.3 per component,
             internal Plummer velocities of the cluster's own mass and radius)
             plus a uniform background of 5% of the particles in the unit cube
             at rest. Total mass 1 in equal-mass particles.
"""
from __future__ import annotations

import math

import numpy as np


def plummer(n: int, seed, rmax: float = 10.0):
    """Plummer sphere (G = M = a = 1) with the inverse-CDF radius capped at rmax.
    `seed` is anything numpy.random.default_rng accepts."""
    rng = np.random.default_rng(seed)
    r = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        u = rng.random(todo.size)
        u = np.where(u == 0, 0.5, u)
        rr = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        ok = rr <= rmax
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    q = np.empty(n)
    todo = np.arange(n)
    pmax = math.sqrt(7.0) * 686 / 19683  # max of q^2 (1 - q^2)^3.5, at q^2 = 2/9
    while todo.size:
        x1, x2 = rng.random(todo.size), rng.random(todo.size)
        ok = pmax * x1 < x2 * x2 * (1 - x2 * x2) ** 3.5
        q[todo[ok]] = x2[ok]
        todo = todo[~ok]
    ve = math.sqrt(2.0) * (1.0 + r * r) ** -0.25

    def iso(norm, a, b):
        z = (1 - 2 * a) * norm
        w = np.sqrt(np.maximum(norm * norm - z * z, 0.0))
        return np.stack([z, w * np.cos(2 * np.pi * b), w * np.sin(2 * np.pi * b)], axis=1)

    x = iso(r, rng.random(n), rng.random(n))
    v = iso(q * ve, rng.random(n), rng.random(n))
    return np.ascontiguousarray(x), np.ascontiguousarray(v)


def uniform(n: int, seed=1):
    """Uniform in [0, 1)^3, zero velocities."""
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(rng.random((n, 3))), np.zeros((n, 3))


CLUSTERS = 8
BACKGROUND_FRACTION = 0.05


def clustered(n: int, seed: int = 4, clusters: int = CLUSTERS, background: float = BACKGROUND_FRACTION):
    """Adaptive-depth stress workload (module docstring). Particles are laid
    out cluster by cluster (cluster k holds its share of the non-background
    particles, the first (n - n_bg) % clusters clusters one more), then the
    background. Returns (x, v, info) with info = {"centres", "radii", "bulk",
    "sizes", "background"}."""
    rng = np.random.default_rng(seed)
    n_bg = int(round(background * n))
    n_cl = n - n_bg
    sizes = np.full(clusters, n_cl // clusters, dtype=np.int64)
    sizes[: n_cl % clusters] += 1
    centres = rng.random((clusters, 3))
    radii = rng.uniform(0.01, 0.1, clusters)
    bulk = rng.normal(0.0, 0.3, (clusters, 3))
    x = np.empty((n, 3))
    v = np.empty((n, 3))
    o = 0
    for k in range(clusters):
        m = int(sizes[k])
        xc, vc = plummer(m, [seed, k])
        mass = m / n  # G = 1, total mass 1 in equal-mass particles
        x[o:o + m] = centres[k] + radii[k] * xc
        v[o:o + m] = bulk[k] + math.sqrt(mass / radii[k]) * vc
        o += m
    x[o:] = rng.random((n_bg, 3))
    v[o:] = 0.0
    info = {"centres": centres, "radii": radii, "bulk": bulk, "sizes": sizes, "background": n_bg}
    return x, v, info
