"""Nonlinear Q1 hexahedra on the tensor-product path (the nonlinear requests of the serving loop).

FP64: <= 1e-12 per entry (floor 1e-3 of the largest entry).  FP32 Jacobian: <= 5e-5 on that scale: the
entries are 32-term FP32 dot products whose terms cancel (the rounding bound is 32 * 2^-24 of the sum of
the absolute terms, which for the smallest entries near the floor is ~20x the entry itself).
"""
import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem
from tests.test_gpu_assembly_parity import TOL64, scaled_err


@pytest.mark.gpu
@pytest.mark.parametrize("n", [(3, 4, 2), (1, 1, 1), (6, 5, 4)])
@pytest.mark.parametrize("fp32", [False, True])
def test_q1_nonlinear_tensor_path_matches_oracle(cuda, n, fp32):
    from mrhyde_gb300 import AssemblyManager

    cfg = dict(dim=3, order=1, n=n, kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=3,
               lo=(0.0, -0.5, 0.0), hi=(1.0, 0.5, 2.0))
    O = oracle_problem(cfg)
    u = np.random.default_rng(60).uniform(0.0, 0.5, O.ndof)
    ro, Jo = O.assemble(u)
    G = gpu_problem(cfg)
    assert G.info.path == 3
    A = AssemblyManager(G)
    r, J = G.new_vector(), G.new_matrix_values(fp32=fp32)
    A.assembleJacRes(torch.tensor(u, device="cuda"), r, J, fp32_jacobian=fp32, overwrite=True)
    assert scaled_err(r.cpu().numpy(), ro) <= TOL64
    assert scaled_err(J.cpu().numpy(), Jo) <= (5e-5 if fp32 else TOL64)
