"""Jacobian and residual of the GPU kernels against the oracle on the same seeded inputs.

Tolerance (FP64 mode): |a - b| <= 1e-12 * max(|b|, 1e-3 * max|b|) per entry -- relative, with a floor
at 1e-3 of the largest entry so that entries that cancel to round-off (e.g. the edge couplings of a
cube cell, exactly zero in exact arithmetic) are compared on the matrix's scale.
Mixed mode (FP32 Jacobian): 2e-6 on the same scale; its FP64 residual keeps the 1e-12 bound.
"""
import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem, perturbed_vertices

TOL64 = 1e-12
TOL32 = 2e-6


def scaled_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = np.max(np.abs(b)) if b.size else 1.0
    scale = np.maximum(np.abs(b), 1e-3 * m)
    scale[scale == 0] = 1.0
    return float(np.max(np.abs(a - b) / scale))


def _run(cfg, u, force_cell=False, atomic=False, fp32=False, seed_J=None):
    from mrhyde_gb300 import AssemblyManager

    G = gpu_problem(cfg)
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r = torch.zeros(G.info.n_dofs, dtype=torch.float64, device="cuda")
    J = torch.zeros(G.info.nnz, dtype=torch.float32 if fp32 else torch.float64, device="cuda")
    A.assembleJacRes(ud, r, J, fp32_jacobian=fp32, force_cell=force_cell, atomic=atomic)
    torch.cuda.synchronize()
    return G, r.cpu().numpy(), J.cpu().numpy()


def _cfgs():
    rng = np.random.default_rng(11)
    out = []
    for (dim, n, faces, src) in [(2, (32, 32), 15, ("sinprod", 1.0, np.pi)), (2, (7, 3), 1 | 8, ("const", 2.5, 0)),
                                 (3, (6, 5, 4), 3, ("const", 1.0, 0)), (3, (9, 2, 3), 63, ("sinprod", 12 * np.pi ** 2, 2 * np.pi)),
                                 (3, (1, 1, 1), 0, ("const", 1.0, 0)), (3, (17, 3, 2), 16, ("const", -3.0, 0))]:
        ncell = int(np.prod(n))
        out.append(dict(dim=dim, order=1, n=n, lo=(0.0, -1.0, 0.5), hi=(2.0, 0.5, 1.0), kappa=np.exp(0.5 * rng.standard_normal(ncell)),
                        dirichlet_faces=faces, source=src, dirichlet=("const", 0.3)))
    return out


CFGS = _cfgs()
IDS = [f"d{c['dim']}n{'x'.join(map(str, c['n']))}f{c['dirichlet_faces']}" for c in CFGS]


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CFGS, ids=IDS)
@pytest.mark.parametrize("path", ["factored", "cell_colored", "cell_atomic"])
def test_fp64_jacres_matches_oracle(cuda, cfg, path):
    O = oracle_problem(cfg)
    u = np.random.default_rng(5).uniform(-1, 1, O.ndof)
    ro, Jo = O.assemble(u)
    G, r, J = _run(cfg, u, force_cell=path != "factored", atomic=path == "cell_atomic")
    if path == "factored":
        assert G.info.path == 1
    assert scaled_err(J, Jo) <= TOL64
    assert scaled_err(r, ro) <= TOL64


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CFGS[:4], ids=IDS[:4])
@pytest.mark.parametrize("path", ["factored", "cell_colored"])
def test_mixed_fp32_jacobian_fp64_residual(cuda, cfg, path):
    O = oracle_problem(cfg)
    u = np.random.default_rng(6).uniform(-1, 1, O.ndof)
    ro, Jo = O.assemble(u)
    _, r, J = _run(cfg, u, fp32=True, force_cell=path != "factored")
    assert scaled_err(J, Jo) <= TOL32
    assert scaled_err(r, ro) <= TOL64


NONAFFINE = [
    dict(dim=2, order=1, n=(6, 5), kind="thermal", source=("sinprod", 2.0, 1.5), dirichlet_faces=1 | 4),
    dict(dim=3, order=1, n=(4, 3, 3), kind="thermal", source=("const", 1.0, 0.0), dirichlet_faces=3),
    dict(dim=2, order=2, n=(3, 4), kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=1),
    dict(dim=3, order=1, n=(3, 3, 2), kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=3),
    dict(dim=3, order=2, n=(2, 3, 2), kind="diffusion_1pu2", source=("const", 10.0, 0.0), dirichlet_faces=3),
    dict(dim=3, order=2, n=(3, 2, 2), kind="thermal", source=("sinprod", 1.0, 2.0), dirichlet_faces=63),
]


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(NONAFFINE)))
@pytest.mark.parametrize("atomic", [False, True])
def test_per_cell_ad_path_general_geometry_and_physics(cuda, i, atomic):
    cfg = dict(NONAFFINE[i])
    dim, n = cfg["dim"], cfg["n"]
    rng = np.random.default_rng(20 + i)
    cfg["kappa"] = np.exp(0.5 * rng.standard_normal(int(np.prod(n))))
    cfg["vertex_coords"] = perturbed_vertices(dim, n, (0, 0, 0), (1, 1, 1), 0.25, 30 + i)
    O = oracle_problem(cfg)
    u = rng.uniform(0.0, 0.5, O.ndof)
    ro, Jo = O.assemble(u)
    G, r, J = _run(cfg, u, atomic=atomic)
    # thermal Q1 cells (quadrilaterals and hexahedra) take the stored-geometry row gather unless the atomic
    # AD scatter is asked for
    stored = cfg["order"] == 1 and cfg["kind"] == "thermal"
    assert G.info.path == (4 if stored else 2)
    assert scaled_err(J, Jo) <= TOL64
    assert scaled_err(r, ro) <= TOL64


@pytest.mark.gpu
def test_sum_into_semantics_and_residual_only(cuda):
    from mrhyde_gb300 import AssemblyManager

    cfg = CFGS[2]
    G = gpu_problem(cfg)
    A = AssemblyManager(G)
    u = torch.tensor(np.random.default_rng(3).uniform(-1, 1, G.info.n_dofs), device="cuda")
    r1 = torch.zeros(G.info.n_dofs, dtype=torch.float64, device="cuda")
    J1 = torch.zeros(G.info.nnz, dtype=torch.float64, device="cuda")
    A.assembleJacRes(u, r1, J1, overwrite=True)
    r2, J2 = r1.clone(), J1.clone()
    A.assembleJacRes(u, r2, J2)  # sum into: doubles every scattered entry, diagonal of fixed rows stays 1
    d, _ = G.fixed_dofs()
    rp, ci = G.graph()
    diag_slots = []
    dn = d.cpu().numpy()
    rpn, cin = rp.cpu().numpy(), ci.cpu().numpy()
    for row in dn:
        k = rpn[row] + np.searchsorted(cin[rpn[row]:rpn[row + 1]], row)
        diag_slots.append(k)
    expect = 2 * J1.cpu().numpy()
    expect[diag_slots] = 1.0
    np.testing.assert_array_equal(J2.cpu().numpy(), expect)
    np.testing.assert_array_equal(r2.cpu().numpy(), 2 * r1.cpu().numpy())
    r3 = torch.full_like(r1, 7.0)
    A.assembleRes(u, r3, overwrite=True)
    np.testing.assert_array_equal(r3.cpu().numpy(), r1.cpu().numpy())
    J4 = torch.full_like(J1, 3.0)
    A.assembleJac(u, J4, overwrite=True)
    np.testing.assert_array_equal(J4.cpu().numpy(), J1.cpu().numpy())


@pytest.mark.gpu
def test_assembly_is_deterministic(cuda):
    from mrhyde_gb300 import AssemblyManager

    cfg = CFGS[3]
    G = gpu_problem(cfg)
    A = AssemblyManager(G)
    u = torch.tensor(np.random.default_rng(4).uniform(-1, 1, G.info.n_dofs), device="cuda")
    outs = []
    for _ in range(2):
        for cell in (False, True):
            r = torch.zeros(G.info.n_dofs, dtype=torch.float64, device="cuda")
            J = torch.zeros(G.info.nnz, dtype=torch.float64, device="cuda")
            A.assembleJacRes(u, r, J, force_cell=cell)
            outs.append((r.cpu().numpy(), J.cpu().numpy()))
    np.testing.assert_array_equal(outs[0][1], outs[2][1])
    np.testing.assert_array_equal(outs[0][0], outs[2][0])
    np.testing.assert_array_equal(outs[1][1], outs[3][1])  # colored scatter: fixed order, bit-identical
