"""Seeded synthetic elliptic instances for batched solves.

``random_elliptic(seed)`` draws one problem of the batched-instances
workload: -div(D grad u) + C u = f on [0,1]^2 with homogeneous Dirichlet
data, where

  * log D is a sum of 16 Fourier modes cos(2 pi (kx x + ky y) + phase) with
    wavenumbers kx, ky drawn from 1..8 and amplitudes N(0, 0.5^2), clipped
    to [ln 0.1, ln 10], so D lies in [0.1, 10];
  * C is the same mode recipe (an independent draw) squashed into [0, 1]
    by 0.5 (1 + tanh(.));
  * f is a sum of 4 Gaussian bumps with widths U[0.02, 0.1], centres
    U[0.1, 0.9]^2 and amplitudes N(0, 100^2);
  * BaseCells is drawn from {32, 64, 128} and MaxLevels from {2, 3, 4}.

Every instance has a 16x16 coarsest grid on the unit square, so any set of
them can share one batch (equal cell size per level).  The draws use
numpy's PCG64 generator seeded with the instance seed, so an instance is
reproducible on any machine.
"""
from __future__ import annotations

import numpy as np

from .problem import ebProblem


def _modes(rng, n=16, kmax=8, sigma=0.5):
    kx = rng.integers(1, kmax + 1, n)
    ky = rng.integers(1, kmax + 1, n)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    a = rng.normal(0.0, sigma, n)

    def s(X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        out = np.zeros(np.broadcast(X, Y).shape)
        for m in range(n):
            out = out + a[m] * np.cos(2 * np.pi * (kx[m] * X + ky[m] * Y) + ph[m])
        return out
    return s


def random_elliptic(seed):
    """One seeded instance: (problem, option dict)."""
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    logd = _modes(rng)
    cs = _modes(rng)
    w = rng.uniform(0.02, 0.1, 4)
    cx = rng.uniform(0.1, 0.9, 4)
    cy = rng.uniform(0.1, 0.9, 4)
    amp = rng.normal(0.0, 100.0, 4)
    base = int(rng.choice([32, 64, 128]))
    maxlev = int(rng.choice([2, 3, 4]))

    D = lambda X, Y: np.exp(np.clip(logd(X, Y), np.log(0.1), np.log(10.0)))
    C = lambda X, Y: 0.5 * (1 + np.tanh(cs(X, Y)))

    def f(X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        out = np.zeros(np.broadcast(X, Y).shape)
        for b in range(4):
            out = out + amp[b] * np.exp(-((X - cx[b]) ** 2 + (Y - cy[b]) ** 2) / (2 * w[b] ** 2))
        return out

    prob = ebProblem([0, 1, 0, 1], D, C, f, ('dirichlet', 0))
    opts = {'BaseCells': base, 'MaxLevels': maxlev, 'TagThreshold': 1e-2, 'Verbose': 0, 'RelTol': 1e-10}
    return prob, opts


def final_stage(prob, opts_dict, backend, tree=False):
    """ebSolve's solution-driven pipeline (ebSolve.m:38-52) up to, but not
    including, its last ebSolveCycles: returns (flat tables of the hierarchy
    that last solve starts from, the hierarchy after the pipeline).  Every
    earlier stage is solved and tagged on ``backend``."""
    from .options import ebOptions
    from .flat import flatten
    from .solve import ebSolveCycles
    from .tagcluster import tag_cluster
    from . import hierarchy as hier
    opts = ebOptions(opts_dict)
    H = hier.setup(prob, opts, backend, tree=tree)
    while True:
        fl = flatten(H)
        if (H.nlev - H.rootIdx + 1) >= opts.MaxLevels:
            return fl, H
        H = ebSolveCycles(H, backend)
        boxes = tag_cluster(H, backend)
        if boxes.shape[0] == 0:
            return fl, H
        H = hier.add_level(H, boxes, backend)
