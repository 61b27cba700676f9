"""Synthetic inputs of the benchmark configurations (seeded, host-generated, then uploaded).

  C1  steady thermal, unit square, 32x32 Q1 quads, f = sin(pi x) sin(pi y), u = 0 on all sides,
      kappa_c = exp(0.5 g_c), g iid N(0,1)
  C2  steady thermal, unit cube, 128^3 Q1 hexes, f = 1, u = 0 on x = 0 and x = 1,
      kappa_c = exp(0.5 g_c)
  C3  nonlinear diffusion -div((1+u^2) grad u) = 10, unit cube, 64^3 Q2 hexes, u0 iid U(0, 0.1),
      u = 0 on x = 0 and x = 1 (the boundary is not named by the configuration; this is the choice)
  C4  4096 independent steady-thermal Q1 hex problems, per-axis cells U{4..16}, kappa = exp(g),
      Dirichlet data U(-1, 1) on all boundary nodes
  C5  serving stream: Poisson arrivals, cube edge log-uniform in [16, 96], lognormal kappa (sigma 1)

Random numbers come from numpy's PCG64 generator (numpy.random.default_rng(seed)); the same arrays
are handed to the GPU library and to the oracle, so parity does not depend on the generator.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib as L


def lognormal_kappa(ncell: int, seed: int, sigma: float = 0.5) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(sigma * rng.standard_normal(ncell))


def c1(seed: int = 1, n: int = 32):
    kap = lognormal_kappa(n * n, seed, 0.5)
    return dict(dim=2, order=1, n=(n, n), lo=(0.0, 0.0), hi=(1.0, 1.0), kind="thermal",
                source=("sinprod", 1.0, math.pi), kappa=kap, dirichlet_faces=L.MRG_FACE_ALL,
                dirichlet=("const", 0.0))


def c2(seed: int = 2, n: int = 128):
    kap = lognormal_kappa(n ** 3, seed, 0.5)
    return dict(dim=3, order=1, n=(n, n, n), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), kind="thermal",
                source=("const", 1.0, 0.0), kappa=kap, dirichlet_faces=L.MRG_FACE_XLO | L.MRG_FACE_XHI,
                dirichlet=("const", 0.0))


def c3(seed: int = 3, n: int = 64):
    nn = 2 * n + 1
    rng = np.random.default_rng(seed)
    u0 = rng.uniform(0.0, 0.1, nn ** 3)
    cfg = dict(dim=3, order=2, n=(n, n, n), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), kind="diffusion_1pu2",
               source=("const", 10.0, 0.0), kappa=1.0, dirichlet_faces=L.MRG_FACE_XLO | L.MRG_FACE_XHI,
               dirichlet=("const", 0.0))
    return cfg, u0


def c4_sizes(nprob: int = 4096, seed: int = 4):
    rng = np.random.default_rng(seed)
    return rng.integers(4, 17, size=(nprob, 3))


def c4_problem(sizes, k: int, seed: int = 4):
    nx, ny, nz = (int(v) for v in sizes[k])
    rng = np.random.default_rng([seed, k])
    kap = np.exp(rng.standard_normal(nx * ny * nz))
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    dbc = rng.uniform(-1.0, 1.0, nn)
    return dict(dim=3, order=1, n=(nx, ny, nz), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), kind="thermal",
                source=("const", 1.0, 0.0), kappa=kap, dirichlet_faces=L.MRG_FACE_ALL, dirichlet=("node", dbc))
