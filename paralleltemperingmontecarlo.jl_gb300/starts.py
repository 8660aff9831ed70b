"""Seeded synthetic start configurations for the benchmark workloads.

The reference's scripts start from Cambridge-database minima or lattices
(examples/ne13.jl:38-56, scripts/cu55.jl:164-224); the synthetic workloads here
use uniform random clusters, fcc boxes and the Cu55 icosahedron instead.
"""
import numpy as np


def sphere_start(N, radius, min_sep, seed, max_tries=200000):
    """N points uniform in a sphere, no pair closer than min_sep (bohr).

    Random sequential addition with a bounded number of tries; if the packing
    jams, min_sep is relaxed by 5 % and the placement restarts."""
    rng = np.random.default_rng(seed)
    sep = float(min_sep)
    for _ in range(40):
        pos = np.zeros((0, 3))
        tries = 0
        while len(pos) < N and tries < max_tries:
            tries += 1
            v = rng.uniform(-radius, radius, 3)
            if v @ v >= radius * radius:
                continue
            if len(pos) and np.min(np.sum((pos - v) ** 2, 1)) <= sep * sep:
                continue
            pos = np.vstack([pos, v])
        if len(pos) == N:
            return pos
        sep *= 0.95
    raise RuntimeError("cannot place %d atoms in a sphere of radius %g" % (N, radius))


def fcc_box(ncell, a, jitter, seed):
    """4*ncell^3 atoms on an fcc lattice of constant a, centred, with uniform jitter."""
    rng = np.random.default_rng(seed)
    basis = [(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)]
    x = np.array([[(i + b[0]) * a, (j + b[1]) * a, (k + b[2]) * a]
                  for i in range(ncell) for j in range(ncell) for k in range(ncell) for b in basis])
    return x + rng.uniform(-jitter, jitter, x.shape) - ncell * a / 2
