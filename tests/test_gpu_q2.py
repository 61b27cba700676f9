"""Q2 hexahedra on affine cells (C3 kernels): sum-factorised FP64 residual + row-gather Jacobian.

Tolerances: FP64 <= 1e-12 per entry (floor 1e-3 of the largest entry), as for Q1.  FP32 Jacobian
<= 1e-5: each Q2 entry is a 108-term FP32 dot product with cancellation, whose rounding bound is
108 * 2^-24 = 6.4e-6 of the sum of the absolute terms.  The nonlinear form -div((1+u^2) grad u) = f is unpinned by the reference's
goldens; the oracle's AD Jacobian for it is checked against finite differences on the CPU.
"""
import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem
from tests.test_gpu_assembly_parity import TOL64, scaled_err

TOL32_Q2 = 1e-5

Q2CASES = [
    dict(dim=3, order=2, n=(3, 2, 4), kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=3),
    dict(dim=3, order=2, n=(2, 2, 2), kind="diffusion_1pu2", source=("const", -2.0, 0.0), dirichlet_faces=0,
         lo=(0.0, 0.0, -1.0), hi=(2.0, 0.5, 1.0)),
    dict(dim=3, order=2, n=(4, 3, 2), kind="thermal", source=("const", 1.0, 0.0), dirichlet_faces=63),
    dict(dim=3, order=2, n=(1, 1, 1), kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=1),
]


def _cfg(i):
    c = dict(Q2CASES[i])
    rng = np.random.default_rng(40 + i)
    c["kappa"] = np.exp(0.5 * rng.standard_normal(int(np.prod(c["n"]))))
    return c


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(Q2CASES)))
@pytest.mark.parametrize("fp32", [False, True])
def test_q2_fast_path_matches_oracle(cuda, i, fp32):
    from mrhyde_gb300 import AssemblyManager

    cfg = _cfg(i)
    O = oracle_problem(cfg)
    u = np.random.default_rng(50 + i).uniform(0.0, 0.3, O.ndof)
    ro, Jo = O.assemble(u)
    G = gpu_problem(cfg)
    assert G.info.path == 3
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r = G.new_vector()
    J = G.new_matrix_values(fp32=fp32)
    A.assembleJacRes(ud, r, J, fp32_jacobian=fp32, overwrite=True, tensor_cores=False)
    assert scaled_err(r.cpu().numpy(), ro) <= TOL64
    assert scaled_err(J.cpu().numpy(), Jo) <= (TOL32_Q2 if fp32 else TOL64)
    # sum-into and residual-only agree with the fused call
    r2 = G.new_vector()
    A.assembleRes(ud, r2)
    np.testing.assert_allclose(r2.cpu().numpy(), r.cpu().numpy(), rtol=0, atol=0)
    J2 = J.clone()
    A.assembleJac(ud, J2, fp32_jacobian=fp32, tensor_cores=False)
    Jn, J2n = J.cpu().numpy().astype(np.float64), J2.cpu().numpy().astype(np.float64)
    d, _ = G.fixed_dofs()
    rp, ci = G.graph()
    rpn, cin = rp.cpu().numpy(), ci.cpu().numpy()
    diag = [rpn[k] + np.searchsorted(cin[rpn[k]:rpn[k + 1]], k) for k in d.cpu().numpy()]
    expect = 2 * Jn
    expect[diag] = 1.0
    if fp32:
        # the Jacobian-only pass computes its Gauss-point coefficients in FP32 (the fused pass reuses the
        # FP64 residual stages): the same FP32 bound against the oracle, not the same bits
        J3 = G.new_matrix_values(fp32=True)
        A.assembleJac(ud, J3, fp32_jacobian=True, overwrite=True, tensor_cores=False)
        assert scaled_err(J3.cpu().numpy(), Jo) <= TOL32_Q2
        assert scaled_err(J2n, expect) <= TOL32_Q2
    else:
        np.testing.assert_allclose(J2n, expect, rtol=1e-15, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_q2_nonlinear_newton_matches_oracle(cuda, mixed):
    """C3 shape at 4^3 Q2 cells: Newton to 1e-10 on -div((1+u^2) grad u) = 10 from u0 ~ U(0, 0.1)."""
    from mrhyde_gb300 import SolverManager
    from mrhyde_gb300.workloads import c3

    cfg, u0 = c3(seed=3, n=4)
    O = oracle_problem(cfg)
    uo = O.set_dirichlet(u0.copy())
    uo, rc, st = O.newton(uo, nltol=1e-10, maxiter=12, lintol=1e-13)
    assert rc == 0
    G = gpu_problem(cfg)
    S = SolverManager(G, nonlinear_tol=1e-10, max_nonlinear_iters=20, linear_tol=1e-12 if not mixed else 1e-5,
                      mixed_precision=mixed)
    u = torch.tensor(u0, device="cuda")
    res = S.nonlinearSolver(u)
    assert res.rel_residual < 1e-10
    err = np.abs(u.cpu().numpy() - uo).max() / np.abs(uo).max()
    assert err < 1e-9, err


@pytest.mark.gpu
@pytest.mark.parametrize("i", [0, 2, 3])
def test_q2_tensor_core_contractions_match_cuda_cores(cuda, i):
    """tcgen05 3xTF32 Jacobian vs the FP32 CUDA-core Jacobian and the oracle.

    Tolerance 1e-4 on the scaled measure (floor 1e-3 of the largest entry): 3xTF32 products are good to
    ~2^-21, but the tensor cores accumulate 3 x 112 products per entry in their own FP32 order, so two
    FP32-class results differ by a few units of 2^-24 of the sum of |terms|, which for entries that
    cancel down to the floor is ~1e-5..1e-4 of the entry."""
    from mrhyde_gb300 import AssemblyManager

    cfg = _cfg(i)
    O = oracle_problem(cfg)
    u = np.random.default_rng(70 + i).uniform(0.0, 0.3, O.ndof)
    ro, Jo = O.assemble(u)
    G = gpu_problem(cfg)
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r1, J1 = G.new_vector(), G.new_matrix_values(fp32=True)
    r2, J2 = G.new_vector(), G.new_matrix_values(fp32=True)
    A.assembleJacRes(ud, r1, J1, fp32_jacobian=True, overwrite=True, tensor_cores=False)
    A.assembleJacRes(ud, r2, J2, fp32_jacobian=True, overwrite=True, tensor_cores=True)
    assert torch.equal(r1, r2)
    assert scaled_err(J2.cpu().numpy(), J1.cpu().numpy()) <= 1e-4
    assert scaled_err(J2.cpu().numpy(), Jo) <= 1e-4
    # sum-into semantics on the tensor-core path
    J3 = J2.clone()
    A.assembleJac(ud, J3, fp32_jacobian=True, tensor_cores=True)
    d, _ = G.fixed_dofs()
    rp, ci = G.graph()
    rpn, cin = rp.cpu().numpy(), ci.cpu().numpy()
    diag = [rpn[k] + np.searchsorted(cin[rpn[k]:rpn[k + 1]], k) for k in d.cpu().numpy()]
    expect = 2 * J2.cpu().numpy().astype(np.float64)
    expect[diag] = 1.0
    # the Jacobian-only pass computes its Gauss-point coefficients in FP32: same bound, not the same bits
    assert scaled_err(J3.cpu().numpy(), expect) <= 1e-4
