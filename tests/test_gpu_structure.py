"""CSR row pointers, column indices, DOF map and Dirichlet DOF list: bit-exact against the oracle."""
import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem

CASES = [
    dict(dim=2, order=1, n=(32, 32)),
    dict(dim=2, order=1, n=(1, 7), dirichlet_faces=4),
    dict(dim=3, order=1, n=(5, 3, 7), dirichlet_faces=3),
    dict(dim=3, order=1, n=(1, 1, 1)),
    dict(dim=3, order=2, n=(3, 2, 4), dirichlet_faces=1 | 32),
    dict(dim=2, order=2, n=(4, 3), dirichlet_faces=0),
]


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CASES, ids=lambda c: f"d{c['dim']}p{c['order']}n{'x'.join(map(str, c['n']))}")
def test_graph_dofmap_fixed_bit_exact(cuda, cfg):
    G, O = gpu_problem(cfg), oracle_problem(cfg)
    assert (G.info.n_dofs, G.info.n_cells, G.info.nnz, G.info.n_fixed) == (O.ndof, O.ncell, O.nnz, O.nfixed)
    rp, ci = G.graph()
    orp, oci = O.graph()
    assert np.array_equal(rp.cpu().numpy(), orp)
    assert np.array_equal(ci.cpu().numpy(), oci)
    assert np.array_equal(G.dof_map().cpu().numpy(), O.dof_map())
    d, v = G.fixed_dofs()
    od, ov = O.fixed()
    assert np.array_equal(d.cpu().numpy(), od)
    assert np.array_equal(v.cpu().numpy(), ov)


@pytest.mark.gpu
def test_c2_graph_sizes(cuda):
    from mrhyde_gb300 import Problem

    P = Problem(dim=3, order=1, n=(128, 128, 128), dirichlet_faces=3)
    assert P.info.n_dofs == 2146689 and P.info.nnz == 57066625 and P.info.n_fixed == 2 * 129 * 129
    rp, ci = P.graph()
    assert int(rp[-1]) == 57066625
    # sortedness and analytic row lengths at full size (size-independent properties)
    lens = (rp[1:] - rp[:-1]).cpu().numpy()
    assert lens.max() == 27 and lens.min() == 8
    d = ci[1:].to(torch.int64) - ci[:-1].to(torch.int64)
    starts = torch.zeros(P.info.nnz, dtype=torch.bool, device="cuda")
    starts[rp[:-1]] = True
    assert bool(torch.all((d > 0) | starts[1:]))
