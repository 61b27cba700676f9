"""Batched multiscale-subgrid solves (C4) against the oracle, and independence from co-scheduled work.

Each local problem: unit cube, Q1 hexes (per-axis cells given), kappa per cell, f constant, Dirichlet
data on every boundary node.  Solution tolerance: 1e-9 of the solution's max norm (FP64 refinement to
rel. inf-norm residual 1e-10 from an FP32 inner solve); FP32 Jacobian: 2e-6 scaled (as elsewhere).
"""
import numpy as np
import pytest
import torch

from tests.cases import oracle_problem
from tests.test_gpu_assembly_parity import TOL32, scaled_err


def _batch(nprob, lo, hi, seed):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, size=(nprob, 3))
    kaps, dbcs = [], []
    for k in range(nprob):
        nx, ny, nz = sizes[k]
        kaps.append(np.exp(rng.standard_normal(nx * ny * nz)))
        dbcs.append(rng.uniform(-1.0, 1.0, (nx + 1) * (ny + 1) * (nz + 1)))
    return sizes, kaps, dbcs


@pytest.mark.gpu
def test_batch_matches_oracle_per_problem(cuda):
    from mrhyde_gb300.subgrid import SubgridBatch

    sizes, kaps, dbcs = _batch(10, 2, 6, 1)
    B = SubgridBatch(sizes, kaps, dbcs, source=1.0)
    st = B.solve(tol=1e-10, inner_tol=1e-5)
    assert np.all(st[:, 3] == 0) and np.all(st[:, 2] <= 1e-10)
    for k in range(len(sizes)):
        cfg = dict(dim=3, order=1, n=tuple(int(v) for v in sizes[k]), kappa=kaps[k], source=("const", 1.0, 0.0),
                   dirichlet_faces=63, dirichlet=("node", dbcs[k]))
        O = oracle_problem(cfg)
        uo = O.set_dirichlet(np.zeros(O.ndof))
        uo, rc, _ = O.newton(uo, nltol=1e-12, maxiter=4, lintol=1e-14)
        u = B.solution(k).cpu().numpy()
        assert np.abs(u - uo).max() <= 1e-9 * np.abs(uo).max(), k
        # the local FP32 Jacobian, on the problem's canonical graph
        _, Jo = O.assemble(uo)
        o = int(B.nnz_off[k])
        J = B.J[o:o + O.nnz].cpu().numpy()
        assert scaled_err(J, Jo) <= TOL32, k


@pytest.mark.gpu
def test_batch_result_is_the_same_alone_and_in_the_mix(cuda):
    from mrhyde_gb300.subgrid import SubgridBatch

    sizes, kaps, dbcs = _batch(64, 2, 12, 2)
    B = SubgridBatch(sizes, kaps, dbcs)
    B.set_config(512, 1)
    B.solve()
    for k in (0, 17, 63):
        A = SubgridBatch(sizes[k:k + 1], kaps[k:k + 1], dbcs[k:k + 1])
        A.set_config(512, 1)
        A.solve()
        assert torch.equal(A.solution(0), B.solution(k))


@pytest.mark.gpu
def test_batch_autotune_and_c4_size(cuda):
    """4096 problems with per-axis cells U{4..16} (C4): every problem converges to 1e-10."""
    from mrhyde_gb300.subgrid import SubgridBatch
    from mrhyde_gb300.workloads import c4_problem, c4_sizes

    sizes = c4_sizes(4096, seed=4)
    probs = [c4_problem(sizes, k, seed=4) for k in range(len(sizes))]
    B = SubgridBatch(sizes, [p["kappa"] for p in probs], [p["dirichlet"][1] for p in probs], source=1.0)
    cfg = B.autotune()
    assert cfg[0] in (256, 512, 1024)
    st = B.solve()
    assert np.all(st[:, 3] == 0)
    assert np.all(st[:, 2] <= 1e-10)
