"""Thermal assembly on general (non-affine) Q1 hexahedra and quadrilaterals from per-cell geometry stored
at creation.

Checked against the oracle's forward-AD assembly on the same vertex coordinates and against the per-cell
AD kernels of the library (MRG_ASM_FORCE_CELL): FP64 Jacobian 1e-12 per entry (floor 1e-3 of the
largest entry), FP32 Jacobian 2e-6; residuals 1e-12 relative to the size of the row's terms (a residual
entry is a sum of cancelling terms, see test_gpu_fullsize.py) and 1e-10 on the per-entry floor measure.
"""
import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem, perturbed_vertices
from tests.test_gpu_assembly_parity import TOL32, TOL64, scaled_err
from tests.test_gpu_fullsize import term_rel_err, term_scale

CASES = [
    dict(n=(5, 4, 3), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), faces=3, source=("const", 1.0, 0.0), amp=0.25),
    dict(n=(3, 6, 4), lo=(-1.0, 0.5, 0.0), hi=(2.0, 1.0, 0.4), faces=63, source=("sinprod", 3.0, 2.0), amp=0.3),
    dict(n=(7, 2, 5), lo=(0.0, 0.0, 0.0), hi=(0.7, 0.2, 0.5), faces=16 | 2, source=("const", -2.0, 0.0), amp=0.2),
    dict(n=(1, 1, 1), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), faces=0, source=("const", 1.0, 0.0), amp=0.0),
    dict(n=(24, 20, 16), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), faces=3, source=("sinprod", 1.0, 3.0), amp=0.25),
    # quadrilaterals
    dict(n=(5, 4), lo=(0.0, 0.0), hi=(1.0, 1.0), faces=1 | 4, source=("sinprod", 2.0, 1.5), amp=0.25),
    dict(n=(3, 7), lo=(-1.0, 0.5), hi=(2.0, 1.0), faces=15, source=("const", -1.0, 0.0), amp=0.3),
    dict(n=(1, 1), lo=(0.0, 0.0), hi=(1.0, 1.0), faces=0, source=("const", 1.0, 0.0), amp=0.0),
    dict(n=(90, 70), lo=(0.0, 0.0), hi=(1.0, 0.6), faces=2, source=("sinprod", 1.0, 3.0), amp=0.25),
]


def _cfg(i):
    c = CASES[i]
    dim = len(c["n"])
    rng = np.random.default_rng(300 + i)
    return dict(dim=dim, order=1, n=c["n"], lo=c["lo"], hi=c["hi"], kind="thermal", source=c["source"],
                kappa=np.exp(0.5 * rng.standard_normal(int(np.prod(c["n"])))), dirichlet_faces=c["faces"],
                dirichlet=("const", 0.25),
                vertex_coords=perturbed_vertices(dim, c["n"], c["lo"], c["hi"], c["amp"], 310 + i))


def _oracle(cfg, u):
    O = oracle_problem(cfg)
    ro, Jo = O.assemble(u)
    b, _ = O.assemble(np.zeros(O.ndof), jac=False)
    return O, ro, Jo, term_scale(O, Jo, u, b)


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(CASES)))
def test_stored_geometry_matches_oracle(cuda, i):
    from mrhyde_gb300 import AssemblyManager

    cfg = _cfg(i)
    G = gpu_problem(cfg)
    assert G.info.path == 4
    u = np.random.default_rng(320 + i).uniform(-1.0, 1.0, G.info.n_dofs)
    O, ro, Jo, s = _oracle(cfg, u)
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r, J = G.new_vector(), G.new_matrix_values()
    r.fill_(np.nan)
    J.fill_(np.nan)
    A.assembleJacRes(ud, r, J, overwrite=True)
    Jn, rn = J.cpu().numpy(), r.cpu().numpy()
    assert scaled_err(Jn, Jo) <= TOL64
    assert term_rel_err(rn, ro, s) <= TOL64
    assert scaled_err(rn, ro) <= 1e-10
    # the per-cell AD kernels of the library agree to the same bound
    r2, J2 = G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(ud, r2, J2, force_cell=True)
    assert scaled_err(Jn, J2.cpu().numpy()) <= TOL64
    assert term_rel_err(rn, r2.cpu().numpy(), s) <= TOL64
    # mixed precision: FP32 Jacobian.  Its FP64 residual is, bit for bit, the residual-only pass's on
    # hexahedra (the mixed pass runs it) and the FP64 pass's on quadrilaterals (the same FP64 row, b - J u)
    r3, J3 = G.new_vector(), G.new_matrix_values(fp32=True)
    J3.fill_(np.nan)
    A.assembleJacRes(ud, r3, J3, fp32_jacobian=True, overwrite=True)
    assert scaled_err(J3.cpu().numpy(), Jo) <= TOL32
    r4 = G.new_vector()
    A.assembleRes(ud, r4, overwrite=True)
    assert torch.equal(r3, r4 if cfg["dim"] == 3 else r)
    assert term_rel_err(r4.cpu().numpy(), ro, s) <= TOL64
    if cfg["dim"] == 2:  # on quadrilaterals the FP32 Jacobian is the FP64 one rounded once
        assert torch.equal(J3, J.float())


@pytest.mark.gpu
@pytest.mark.parametrize("i", [0, 6])
def test_stored_geometry_passes_agree_and_sum_into(cuda, i):
    import scipy.sparse as sp

    from mrhyde_gb300 import AssemblyManager

    cfg = _cfg(i)
    G = gpu_problem(cfg)
    A = AssemblyManager(G)
    ud = torch.tensor(np.random.default_rng(5).uniform(-1, 1, G.info.n_dofs), device="cuda")
    r1, J1 = G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(ud, r1, J1, overwrite=True)
    r2 = torch.full_like(r1, 3.0)
    A.assembleRes(ud, r2, overwrite=True)
    # the residual-only pass forms r per cell, the fused FP64 pass from its Jacobian row: the same sum in
    # exact arithmetic, equal to a few ulps of the row's terms
    b = G.new_vector()
    A.assembleRes(torch.zeros_like(ud), b, overwrite=True)
    rp, ci = G.graph()
    Aabs = sp.csr_matrix((np.abs(J1.cpu().numpy()), ci.cpu().numpy(), rp.cpu().numpy()), shape=(G.info.n_dofs,) * 2)
    scale = Aabs @ np.abs(ud.cpu().numpy()) + np.abs(b.cpu().numpy())
    d, _ = G.fixed_dofs()
    scale[d.cpu().numpy()] = 0.0
    assert term_rel_err(r2.cpu().numpy(), r1.cpu().numpy(), scale) <= 1e-14
    J2 = torch.full_like(J1, 5.0)
    A.assembleJac(ud, J2, overwrite=True)
    assert torch.equal(J1, J2)
    r3, J3 = r1.clone(), J1.clone()
    A.assembleJacRes(ud, r3, J3)  # sum-into: every scattered entry doubles, J(d,d) stays 1
    rpn, cin = rp.cpu().numpy(), ci.cpu().numpy()
    diag = [rpn[k] + np.searchsorted(cin[rpn[k]:rpn[k + 1]], k) for k in d.cpu().numpy()]
    expect = 2 * J1.cpu().numpy()
    expect[diag] = 1.0
    np.testing.assert_array_equal(J3.cpu().numpy(), expect)
    np.testing.assert_array_equal(r3.cpu().numpy(), 2 * r1.cpu().numpy())
    # FP32 Jacobian-only pass in sum-into mode (the staged row path): doubles, diagonal of fixed rows 1
    J32 = G.new_matrix_values(fp32=True)
    A.assembleJac(ud, J32, fp32_jacobian=True, overwrite=True)
    J32b = J32.clone()
    A.assembleJac(ud, J32b, fp32_jacobian=True)
    e32 = 2 * J32.cpu().numpy()
    e32[diag] = 1.0
    np.testing.assert_array_equal(J32b.cpu().numpy(), e32)
    # deterministic: a second call of each pass gives the same bits
    r4, J4 = G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(ud, r4, J4, overwrite=True)
    assert torch.equal(r4, r1) and torch.equal(J4, J1)
    r5 = G.new_vector()
    A.assembleRes(ud, r5, overwrite=True)
    assert torch.equal(r5, r2)


@pytest.mark.gpu
@pytest.mark.parametrize("i", [2, 5])
def test_stored_geometry_follows_new_kappa(cuda, i):
    """The stored data is kappa-free: set_kappa after creation changes J and r as in the oracle."""
    from mrhyde_gb300 import AssemblyManager

    cfg = _cfg(i)
    G = gpu_problem(cfg)
    kap2 = np.exp(np.random.default_rng(9).standard_normal(G.info.n_cells))
    G.set_kappa(torch.tensor(kap2, device="cuda"))
    cfg2 = dict(cfg, kappa=kap2)
    u = np.random.default_rng(10).uniform(-1, 1, G.info.n_dofs)
    O, ro, Jo, s = _oracle(cfg2, u)
    A = AssemblyManager(G)
    r, J = G.new_vector(), G.new_matrix_values()
    A.assembleJacRes(torch.tensor(u, device="cuda"), r, J, overwrite=True)
    assert scaled_err(J.cpu().numpy(), Jo) <= TOL64
    assert term_rel_err(r.cpu().numpy(), ro, s) <= TOL64


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_stored_geometry_newton_matches_oracle(cuda, dim):
    """Newton (a linear problem: one step) with Jacobi PCG on a perturbed 12^3 or 40^2 mesh, FP64 and mixed."""
    from mrhyde_gb300 import SolverManager

    n = (12, 12, 12) if dim == 3 else (40, 40)
    ncell = int(np.prod(n))
    cfg = dict(_cfg(0 if dim == 3 else 5), n=n, lo=(0.0,) * dim, hi=(1.0,) * dim,
               kappa=np.exp(0.5 * np.random.default_rng(4).standard_normal(ncell)),
               vertex_coords=perturbed_vertices(dim, n, (0, 0, 0), (1, 1, 1), 0.25, 44))
    O = oracle_problem(cfg)
    uo = O.set_dirichlet(np.zeros(O.ndof))
    uo, rc, _ = O.newton(uo, nltol=1e-10, maxiter=10, lintol=1e-13)
    assert rc == 0
    G = gpu_problem(cfg)
    for mixed in (False, True):
        S = SolverManager(G, nonlinear_tol=1e-10, max_nonlinear_iters=10, linear_tol=1e-12 if not mixed else 1e-5,
                          mixed_precision=mixed)
        u = G.new_vector()
        res = S.nonlinearSolver(u)
        assert res.rel_residual < 1e-10
        assert np.abs(u.cpu().numpy() - uo).max() <= 1e-9 * np.abs(uo).max()
