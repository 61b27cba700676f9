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


def perturbed_vertices(n, amp: float = 0.2, seed: int = 12, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """Vertex coordinates [prod(n_k + 1), len(n)] (x fastest) of a box of len(n) = 2 or 3 axes whose
    interior vertices are moved by up to amp * h per axis (uniform, seeded): non-affine quadrilaterals or
    hexahedra, the general geometry paths."""
    d = len(n)
    rng = np.random.default_rng(seed)
    axes = [np.linspace(lo[k], hi[k], n[k] + 1) for k in range(d)]
    grids = np.meshgrid(*reversed(axes), indexing="ij")  # slowest axis first
    pts = np.stack([grids[d - 1 - k].reshape(-1) for k in range(d)], axis=1)
    idx_grids = np.meshgrid(*[np.arange(n[k] + 1) for k in reversed(range(d))], indexing="ij")
    idx = np.stack([idx_grids[d - 1 - k].reshape(-1) for k in range(d)], axis=1)
    interior = np.all((idx > 0) & (idx < np.array(n)), axis=1)
    h = np.array([(hi[k] - lo[k]) / n[k] for k in range(d)])
    pts[interior] += amp * h * rng.uniform(-1.0, 1.0, (int(interior.sum()), d))
    return np.ascontiguousarray(pts)


def c2_general(seed: int = 2, n: int = 128, amp: float = 0.2):
    """C2 on a mesh of non-affine hexahedra (interior vertices perturbed by up to 0.2 h): the same
    coefficients, source and boundary data as C2, assembled by the general geometry path."""
    cfg = c2(seed=seed, n=n)
    cfg["vertex_coords"] = perturbed_vertices((n, n, n), amp, seed + 10)
    return cfg


def c1_general(seed: int = 1, n: int = 2048, amp: float = 0.2):
    """C1's coefficients, source and boundary data on n^2 non-affine quadrilaterals (interior vertices
    perturbed by up to 0.2 h)."""
    cfg = c1(seed=seed, n=n)
    cfg["vertex_coords"] = perturbed_vertices((n, n), amp, seed + 10, lo=(0.0, 0.0), hi=(1.0, 1.0))
    return cfg


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
