"""Device PCG and Newton against the oracle and the reference's regression goldens."""
import json
import math
import os

import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "regression_goldens.json")))


def _num(s):
    return float(eval(str(s).replace("^", "**"), {"pi": math.pi}))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["3D_verification", "2D_verification"])
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_newton_reproduces_regression_gold(cuda, case, mixed):
    from mrhyde_gb300 import SolverManager

    g = GOLD[case]
    cfg = dict(dim=g["dim"], order=g["order"], n=tuple(g["n"]), quad_order=g["quad_order"],
               source=(g["source"][0], _num(g["source"][1]), _num(g["source"][2])), dirichlet_faces=63 if g["dim"] == 3 else 15)
    G = gpu_problem(cfg)
    S = SolverManager(G, nonlinear_tol=1e-10, max_nonlinear_iters=8, linear_tol=1e-12 if not mixed else 1e-5,
                      mixed_precision=mixed)
    u = G.new_vector()
    res = S.nonlinearSolver(u)
    assert res.rel_residual < 1e-10
    O = oracle_problem(cfg)
    l2, h1 = O.errors(u.cpu().numpy(), _num(g["exact"][0]), _num(g["exact"][1]))
    assert float(f"{l2:.6g}") == g["l2_T"]
    if "l2_gradT" in g:
        assert float(f"{h1:.6g}") == g["l2_gradT"]


@pytest.mark.gpu
def test_pcg_matches_oracle_pcg(cuda):
    from mrhyde_gb300 import AssemblyManager, SolverManager
    from mrhyde_gb300.workloads import c1

    cfg = c1(seed=3)
    G, O = gpu_problem(cfg), oracle_problem(cfg)
    A, S = AssemblyManager(G), SolverManager(G)
    u = G.new_vector()
    r, J = G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x = G.new_vector()
    res = S.PCG(J, r, x, tol=1e-10, maxiter=5000)
    ro, Jo = O.assemble(np.zeros(O.ndof))
    xo, ito, rro = O.pcg(Jo, ro, tol=1e-10)
    assert abs(res.iterations - ito) <= 2
    assert res.rel_residual <= 1e-10
    np.testing.assert_allclose(x.cpu().numpy(), xo, rtol=0, atol=1e-9 * np.abs(xo).max())


@pytest.mark.gpu
def test_c1_end_to_end_fp64_and_mixed_agree_with_oracle(cuda):
    """C1: 32^2 Q1 quads, kappa = exp(0.5 g), f = sin(pi x) sin(pi y): Newton+PCG to 1e-10."""
    from mrhyde_gb300 import SolverManager
    from mrhyde_gb300.workloads import c1

    cfg = c1(seed=1)
    O = oracle_problem(cfg)
    uo = O.set_dirichlet(np.zeros(O.ndof))
    uo, rc, st = O.newton(uo, nltol=1e-10, maxiter=6, lintol=1e-12)
    assert rc == 0
    for mixed in (False, True):
        G = gpu_problem(cfg)
        S = SolverManager(G, nonlinear_tol=1e-10, max_nonlinear_iters=8, linear_tol=1e-12 if not mixed else 1e-5,
                          mixed_precision=mixed)
        u = G.new_vector()
        res = S.nonlinearSolver(u)
        assert res.rel_residual < 1e-10
        err = np.abs(u.cpu().numpy() - uo).max() / np.abs(uo).max()
        assert err < 1e-9, (mixed, err)


@pytest.mark.gpu
def test_spmv_matches_oracle(cuda):
    from mrhyde_gb300 import AssemblyManager, SolverManager

    rng = np.random.default_rng(9)
    n = (5, 4, 3)
    cfg = dict(dim=3, order=1, n=n, kappa=np.exp(rng.standard_normal(60)), dirichlet_faces=5)
    G, O = gpu_problem(cfg), oracle_problem(cfg)
    A, S = AssemblyManager(G), SolverManager(G)
    u = G.new_vector()
    r, J = G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x = rng.standard_normal(G.info.n_dofs)
    y = G.new_vector()
    S.apply(J, torch.tensor(x, device="cuda"), y)
    yo = O.spmv(J.cpu().numpy(), x)
    np.testing.assert_allclose(y.cpu().numpy(), yo, rtol=1e-13, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("fp32", [False, True])
def test_bicgstab_solves_nonsymmetric_jacobian(cuda, fp32):
    """The 1+u^2 Jacobian is nonsymmetric; BiCGStab (the reference's Belos BiCGStab option) solves it."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    from mrhyde_gb300 import AssemblyManager, SolverManager

    cfg = dict(dim=3, order=1, n=(10, 9, 8), kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=3)
    G, O = gpu_problem(cfg), oracle_problem(cfg)
    u = np.random.default_rng(81).uniform(0.0, 0.8, G.info.n_dofs)
    ro, Jo = O.assemble(u)
    rp, ci = O.graph()
    A = sp.csr_matrix((Jo, ci, rp), shape=(O.ndof, O.ndof))
    assert abs(A - A.T).max() > 1e-3 * abs(A).max()  # genuinely nonsymmetric
    xo = spl.spsolve(A.tocsc(), ro)
    Am, S = AssemblyManager(G), SolverManager(G)
    r, J = G.new_vector(), G.new_matrix_values(fp32=fp32)
    Am.assembleJacRes(torch.tensor(u, device="cuda"), r, J, fp32_jacobian=fp32, overwrite=True)
    x = G.new_vector()
    tol = 1e-5 if fp32 else 1e-11
    res = S.BiCGStab(J, r, x, tol=tol, maxiter=5000)
    assert res.rel_residual <= tol
    err = np.abs(x.cpu().numpy() - xo).max() / np.abs(xo).max()
    assert err < (1e-3 if fp32 else 1e-8), err


@pytest.mark.gpu
def test_bicgstab_matches_pcg_on_spd_system(cuda):
    from mrhyde_gb300 import AssemblyManager, SolverManager
    from mrhyde_gb300.workloads import c1

    G = gpu_problem(c1(seed=5))
    A, S = AssemblyManager(G), SolverManager(G)
    u, r, J = G.new_vector(), G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x1, x2 = G.new_vector(), G.new_vector()
    S.PCG(J, r, x1, tol=1e-12, maxiter=5000)
    S.BiCGStab(J, r, x2, tol=1e-12, maxiter=5000)
    np.testing.assert_allclose(x2.cpu().numpy(), x1.cpu().numpy(), rtol=0, atol=1e-9 * x1.abs().max().item())


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_newton_nonlinear_uses_bicgstab_and_converges_fast(cuda, mixed):
    from mrhyde_gb300 import SolverManager
    from mrhyde_gb300.workloads import c3

    cfg, u0 = c3(seed=3, n=8)
    G = gpu_problem(cfg)
    S = SolverManager(G, nonlinear_tol=1e-10, max_nonlinear_iters=25, linear_tol=1e-3 if mixed else 1e-10,
                      linear_maxiter=20000, mixed_precision=mixed)
    u = torch.tensor(u0, device="cuda")
    res = S.nonlinearSolver(u)
    assert res.rel_residual < 1e-10
    assert res.iterations < 200 * res.outer_iterations
