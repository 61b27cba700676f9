"""Face boundary terms on the GPU (Neumann and weakly imposed Dirichlet data) against the oracle, on box
cells and on general (non-affine) cells, whose side weights, normals and element sizes come from each face
cell's own geometry.

Reference: thermal::boundaryResidual (src/physics/thermal.cpp:170-260) in the boundary workset loop of
assembleJacRes (src/managers/assembly/assemblyManager_jacres.hpp:485-603).  Same seeded inputs and the
same boundary data at the side points on both sides; tolerances as in test_gpu_assembly_parity (FP64
1e-12 on the scaled entry error; FP32 Jacobians at the tolerance of their volume path).  The 2D_mixed_bcs
regression gold (Neumann data on two faces) is reproduced through the device Newton.
"""
import json
import math
import os

import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem
from tests.test_gpu_assembly_parity import TOL64, scaled_err

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "regression_goldens.json")))

# (cfg, {face: kind}, FP32 tolerance of the volume path)
CASES = [
    (dict(dim=2, order=1, n=(9, 7), lo=(0.0, -1.0, 0.0), hi=(2.0, 0.5, 1.0), dirichlet_faces=1, source=("const", 2.0, 0.0)),
     {2: "neumann", 3: "weak_dirichlet", 1: "weak_dirichlet"}, 2e-6),
    (dict(dim=3, order=1, n=(5, 4, 3), lo=(0.0, -1.0, 0.5), hi=(2.0, 0.5, 1.0), dirichlet_faces=1,
          source=("sinprod", 3.0, 2.0)), {5: "neumann", 2: "weak_dirichlet"}, 2e-6),
    (dict(dim=3, order=1, n=(4, 3, 3), kind="diffusion_1pu2", dirichlet_faces=1, source=("const", 10.0, 0.0)),
     {1: "weak_dirichlet", 3: "neumann"}, 5e-5),
    (dict(dim=3, order=2, n=(3, 3, 2), kind="diffusion_1pu2", dirichlet_faces=1, source=("const", 10.0, 0.0)),
     {4: "weak_dirichlet", 2: "neumann"}, 1e-4),
    (dict(dim=2, order=2, n=(5, 4), dirichlet_faces=0, source=("const", 1.0, 0.0)),
     {0: "weak_dirichlet", 1: "weak_dirichlet", 2: "neumann", 3: "weak_dirichlet"}, 2e-6),
]
IDS = [f"d{c['dim']}p{c['order']}{c.get('kind', 'thermal')[:4]}" for c, _, _ in CASES]
ORC_KIND = {"neumann": 1, "weak_dirichlet": 2}


def _data(xyz, face):
    return np.sin(1.7 * xyz[:, 0] + 0.3 * face) * np.cos(2.3 * xyz[:, 1]) + 0.25 * xyz[:, 2] + 0.1 * face


def _moved_vertices(dim, n, lo, hi, amp, seed):
    """Vertex grid of a box with every vertex moved by up to amp * h per axis: non-affine cells whose
    boundary faces are neither flat nor axis-aligned (side measures and normals differ per face cell)."""
    rng = np.random.default_rng(seed)
    axes = [np.linspace(lo[k], hi[k], n[k] + 1) for k in range(dim)]
    grids = np.meshgrid(*reversed(axes), indexing="ij")  # slowest axis first
    pts = np.stack([grids[dim - 1 - k].reshape(-1) for k in range(dim)], axis=1)
    h = np.array([(hi[k] - lo[k]) / n[k] for k in range(dim)])
    pts += amp * h * rng.uniform(-1, 1, pts.shape)
    return np.ascontiguousarray(pts)


def _setup(cfg, faces, seed, general=False):
    rng = np.random.default_rng(seed)
    ncell = int(np.prod(cfg["n"]))
    c = dict(cfg)
    if c.get("kind", "thermal") == "thermal":
        c["kappa"] = np.exp(0.5 * rng.standard_normal(ncell))
    if general:
        lo = c.get("lo", (0.0, 0.0, 0.0))
        hi = c.get("hi", (1.0, 1.0, 1.0))
        c["vertex_coords"] = _moved_vertices(c["dim"], c["n"], lo, hi, 0.2, seed + 100)
    G, O = gpu_problem(c), oracle_problem(c)
    for face, kind in faces.items():
        xo = O.side_points(face)
        xg = G.side_points(face)
        np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-13)
        g = _data(xo, face)
        O.set_face_bc(face, ORC_KIND[kind], g)
        G.set_face_bc(face, kind, g)
    u = rng.uniform(0.0, 0.4, O.ndof)
    return G, O, u


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("fp32", [False, True])
def test_face_terms_match_oracle(cuda, case, fp32):
    from mrhyde_gb300 import AssemblyManager

    cfg, faces, tol32 = case
    G, O, u = _setup(cfg, faces, 5)
    ro, Jo = O.assemble(u)
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r, J = G.new_vector(), G.new_matrix_values(fp32=fp32)
    A.assembleJacRes(ud, r, J, fp32_jacobian=fp32, overwrite=True)
    torch.cuda.synchronize()
    assert scaled_err(r.cpu().numpy(), ro) <= TOL64
    assert scaled_err(J.cpu().numpy(), Jo) <= (tol32 if fp32 else TOL64)
    # residual-only assembly sees the same boundary terms
    r2 = G.new_vector()
    A.assembleRes(ud, r2, overwrite=True)
    torch.cuda.synchronize()
    assert scaled_err(r2.cpu().numpy(), ro) <= TOL64


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("fp32", [False, True])
def test_face_terms_general_geometry_match_oracle(cuda, case, fp32):
    """Perturbed interior vertices: the volume terms take the stored-geometry or the per-cell AD path, the
    face terms each face cell's own weights, normal derivatives and element size."""
    from mrhyde_gb300 import AssemblyManager

    cfg, faces, tol32 = case
    G, O, u = _setup(cfg, faces, 7, general=True)
    ro, Jo = O.assemble(u)
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r, J = G.new_vector(), G.new_matrix_values(fp32=fp32)
    A.assembleJacRes(ud, r, J, fp32_jacobian=fp32, overwrite=True)
    torch.cuda.synchronize()
    assert scaled_err(r.cpu().numpy(), ro) <= TOL64
    # FP32: the stored-geometry Jacobian forms its products in FP32 and the face terms add one more FP32
    # rounding, each relative to terms that cancel on distorted cells (measured at most 4.0e-6 over the
    # cases, box cells up to 3.7e-5)
    assert scaled_err(J.cpu().numpy(), Jo) <= (max(tol32, 1e-5) if fp32 else TOL64)
    r2 = G.new_vector()
    A.assembleRes(ud, r2, overwrite=True)
    torch.cuda.synchronize()
    assert scaled_err(r2.cpu().numpy(), ro) <= TOL64
    # the boundary terms are there: without them the residual differs
    for face in faces:
        G.set_face_bc(face, "none")
    r3 = G.new_vector()
    A.assembleRes(ud, r3, overwrite=True)
    torch.cuda.synchronize()
    assert scaled_err(r3.cpu().numpy(), ro) > 1e-6


@pytest.mark.gpu
def test_face_terms_on_cell_path(cuda):
    from mrhyde_gb300 import AssemblyManager

    cfg, faces, _ = CASES[1]
    G, O, u = _setup(cfg, faces, 9)
    ro, Jo = O.assemble(u)
    ud = torch.tensor(u, device="cuda")
    r, J = G.new_vector(), G.new_matrix_values()
    AssemblyManager(G).assembleJacRes(ud, r, J, overwrite=True, force_cell=True)
    torch.cuda.synchronize()
    assert scaled_err(r.cpu().numpy(), ro) <= TOL64
    assert scaled_err(J.cpu().numpy(), Jo) <= TOL64


@pytest.mark.gpu
def test_face_bc_argument_checks(cuda):
    from mrhyde_gb300._lib import MrgError
    from tests.cases import perturbed_vertices

    G = gpu_problem(dict(dim=2, order=1, n=(4, 4), dirichlet_faces=1))
    with pytest.raises(MrgError):
        G.set_face_bc(0, "neumann")          # strong Dirichlet face
    with pytest.raises(MrgError):
        G.set_face_bc(7, "neumann")          # no such face in 2-D
    G.set_face_bc(1, "neumann")              # zero data
    G.set_face_bc(1, "none")
    H = gpu_problem(dict(dim=2, order=1, n=(3, 3), dirichlet_faces=1,
                         vertex_coords=perturbed_vertices(2, (3, 3), (0, 0, 0), (1, 1, 1), 0.1, 2)))
    with pytest.raises(MrgError):
        H.set_face_bc(0, "weak_dirichlet")   # strong Dirichlet face, non-affine cells
    H.set_face_bc(1, "neumann")              # non-affine cells: per-cell side geometry
    H.set_face_bc(1, "none")


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_newton_reproduces_mixed_bcs_gold(cuda, mixed):
    from mrhyde_gb300 import SolverManager
    from tests.test_oracle_goldens import side_values

    g = GOLD["2D_mixed_bcs"]
    cfg = dict(dim=2, order=1, n=tuple(g["n"]), quad_order=g["quad_order"], dirichlet_faces=g["dirichlet_faces"],
               source=("sinprod", 8 * math.pi ** 2, 2 * math.pi))
    G = gpu_problem(cfg)
    for face, expr in g["neumann"]:
        G.set_face_bc(face, "neumann", side_values(G.side_points(face), expr))
    S = SolverManager(G, nonlinear_tol=1e-10, max_nonlinear_iters=8, linear_tol=1e-12 if not mixed else 1e-5,
                      mixed_precision=mixed)
    u = G.new_vector()
    res = S.nonlinearSolver(u)
    assert res.rel_residual < 1e-10
    l2, _ = oracle_problem(cfg).errors(u.cpu().numpy(), 1.0, 2 * math.pi)
    assert float(f"{l2:.6g}") == g["l2_T"]
