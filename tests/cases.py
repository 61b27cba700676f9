"""Shared helpers for the parity tests: build the same problem in the GPU library and in the oracle."""
from __future__ import annotations

import numpy as np

FACE_BITS = {"xlo": 1, "xhi": 2, "ylo": 4, "yhi": 8, "zlo": 16, "zhi": 32}


def oracle_problem(cfg):
    from oracle.oracle import OracleProblem

    kind = {"thermal": 0, "diffusion_1pu2": 1}[cfg.get("kind", "thermal")]
    kw = dict(dim=cfg["dim"], order=cfg["order"], n=cfg["n"], lo=cfg.get("lo", (0, 0, 0)), hi=cfg.get("hi", (1, 1, 1)),
              kind=kind, source=cfg.get("source", ("const", 1.0, 0.0)), kappa=cfg.get("kappa", 1.0),
              dirichlet_faces=cfg.get("dirichlet_faces", 63), dirichlet=cfg.get("dirichlet", ("const", 0.0)),
              quad_order=cfg.get("quad_order", 0), workset_size=cfg.get("workset_size", 0),
              vertex_coords=cfg.get("vertex_coords"))
    return OracleProblem(**kw)


def gpu_problem(cfg):
    from mrhyde_gb300 import Problem

    kw = {k: v for k, v in cfg.items() if k in ("dim", "order", "n", "lo", "hi", "kind", "source", "kappa",
                                                "dirichlet_faces", "dirichlet", "quad_order", "vertex_coords")}
    return Problem(**kw)


def perturbed_vertices(dim, n, lo, hi, amp, seed):
    """Vertex grid of a box with interior vertices moved by up to amp*h (non-affine cells)."""
    rng = np.random.default_rng(seed)
    axes = [np.linspace(lo[k], hi[k], n[k] + 1) for k in range(dim)]
    grids = np.meshgrid(*axes, indexing="ij")
    pts = np.stack([g.transpose(*reversed(range(dim))).reshape(-1) for g in grids], axis=1)
    h = np.array([(hi[k] - lo[k]) / n[k] for k in range(dim)])
    idx = np.stack(np.meshgrid(*[np.arange(n[k] + 1) for k in range(dim)], indexing="ij"), -1)
    idx = idx.transpose(*reversed(range(dim)), dim).reshape(-1, dim)
    interior = np.all((idx > 0) & (idx < np.array(n[:dim])), axis=1)
    pts[interior] += amp * h * rng.uniform(-1, 1, (interior.sum(), dim))
    return np.ascontiguousarray(pts)


def rel_err(a, b, floor_frac=1e-14):
    """max |a-b| / max(|b|_inf * floor_frac-scaled entry magnitude) -- relative per entry with a floor."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.abs(b), floor_frac * np.max(np.abs(b)) if b.size else 1.0)
    scale = np.where(scale == 0, 1.0, scale)
    return float(np.max(np.abs(a - b) / scale)) if a.size else 0.0
