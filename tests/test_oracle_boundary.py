"""Boundary terms of the oracle (reference src/physics/thermal.cpp:170-260).

* the AD Jacobian of the Neumann + weak-Dirichlet (Nitsche) terms matches central differences of the
  residual, on non-affine cells, for both physics forms;
* for the linear thermal form the symmetric Nitsche terms (form_param = 1) keep J symmetric;
* weak Dirichlet on every face converges to the manufactured solution at second order in L2 (Q1),
  close to the strongly imposed condition's error;
* the side points and weights integrate the face measure exactly.
The 2D_mixed_bcs regression gold (Neumann data) is pinned in test_oracle_goldens.py.
"""
import math

import numpy as np
import pytest

from tests.cases import oracle_problem, perturbed_vertices
from tests.test_oracle_properties import _dense


def _face_data(P, face, f):
    xyz = P.side_points(face)
    return f(xyz)


@pytest.mark.parametrize("dim,order,kind", [(2, 1, "thermal"), (2, 2, "diffusion_1pu2"), (3, 1, "thermal"),
                                            (3, 1, "diffusion_1pu2")])
def test_boundary_jacobian_matches_finite_differences(dim, order, kind):
    n = (3, 2, 2)[:dim]
    rng = np.random.default_rng(11)
    ncell = int(np.prod(n))
    cfg = dict(dim=dim, order=order, n=n, kind=kind, source=("sinprod", 3.0, 2.0),
               kappa=np.exp(rng.standard_normal(ncell)), dirichlet_faces=1,
               vertex_coords=perturbed_vertices(dim, n, (0, 0, 0), (1, 1, 1), 0.2, 5))
    P = oracle_problem(cfg)
    P.set_face_bc(1, 2, _face_data(P, 1, lambda x: np.sin(3 * x[:, 1]) + 0.5))       # weak Dirichlet on x+
    P.set_face_bc(2, 1, _face_data(P, 2, lambda x: np.cos(2 * x[:, 0]) - 0.3))       # Neumann on y-
    P.set_face_bc(3, 2, _face_data(P, 3, lambda x: x[:, 0] * x[:, 0]))               # weak Dirichlet on y+
    u = rng.uniform(0.0, 1.0, P.ndof)
    r, J = P.assemble(u)
    A = _dense(P, J)
    fixed, _ = P.fixed()
    free = np.setdiff1d(np.arange(P.ndof), fixed)
    eps = 1e-6
    for j in range(P.ndof):
        up, um = u.copy(), u.copy()
        up[j] += eps
        um[j] -= eps
        rp_, _ = P.assemble(up, jac=False)
        rm_, _ = P.assemble(um, jac=False)
        col = -(rp_ - rm_) / (2 * eps)
        np.testing.assert_allclose(A[free, j], col[free], rtol=1e-6, atol=1e-8 * np.abs(A).max())


def test_nitsche_jacobian_symmetric_for_linear_form():
    rng = np.random.default_rng(3)
    n = (4, 3)
    P = oracle_problem(dict(dim=2, order=1, n=n, kappa=np.exp(rng.standard_normal(12)), dirichlet_faces=0))
    for face in range(4):
        P.set_face_bc(face, 2, np.zeros(len(P.side_points(face))))
    _, J = P.assemble(np.zeros(P.ndof))
    A = _dense(P, J)
    np.testing.assert_allclose(A, A.T, rtol=0, atol=1e-13 * np.abs(A).max())
    # with epen = 10 / h the operator stays positive definite here
    assert np.linalg.eigvalsh(0.5 * (A + A.T)).min() > 0


def _weak_error(nc):
    P = oracle_problem(dict(dim=2, order=1, n=(nc, nc), quad_order=2, dirichlet_faces=0,
                            source=("sinprod", 8 * math.pi ** 2, 2 * math.pi)))
    for face in range(4):
        P.set_face_bc(face, 2, np.zeros(len(P.side_points(face))))
    u, rc, _ = P.newton(np.zeros(P.ndof), nltol=1e-12, maxiter=4, lintol=1e-13, linmaxiter=100000, nthreads=2)
    assert rc == 0
    return P.errors(u, 1.0, 2 * math.pi)[0]


def test_weak_dirichlet_converges_at_second_order():
    e20, e40 = _weak_error(20), _weak_error(40)
    assert 3.6 < e20 / e40 < 4.4, (e20, e40)
    strong = 0.00102776  # 2D_verification gold (strong u = 0 on all faces, same mesh)
    assert 0.5 < e40 / strong < 2.0, e40


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_side_points_cover_each_face(dim, order):
    n = (3, 4, 2)[:dim]
    P = oracle_problem(dict(dim=dim, order=order, n=n, lo=(0.5, -1.0, 2.0), hi=(1.5, 1.0, 2.5), dirichlet_faces=0))
    lo, hi = np.array((0.5, -1.0, 2.0)), np.array((1.5, 1.0, 2.5))
    for face in range(2 * dim):
        a = face // 2
        xyz = P.side_points(face)
        assert np.allclose(xyz[:, a], hi[a] if face % 2 else lo[a])
        for k in range(dim):
            if k != a:
                assert (xyz[:, k] > lo[k]).all() and (xyz[:, k] < hi[k]).all()
        # a Neumann flux g = 1 contributes -measure(face) to the residual sum (int phi = measure)
        Q = oracle_problem(dict(dim=dim, order=order, n=n, lo=(0.5, -1.0, 2.0), hi=(1.5, 1.0, 2.5),
                                dirichlet_faces=0, source=("const", 0.0, 0.0)))
        Q.set_face_bc(face, 1, np.ones(len(xyz)))
        r, _ = Q.assemble(np.zeros(Q.ndof), jac=False)
        meas = np.prod([hi[k] - lo[k] for k in range(dim) if k != a])
        assert abs(r.sum() - meas) < 1e-12 * max(1.0, meas), (face, r.sum(), meas)
