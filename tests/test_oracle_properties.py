"""Self-consistency of the oracle: AD Jacobian vs finite differences, graph layout, threading."""
import numpy as np
import pytest

from tests.cases import oracle_problem, perturbed_vertices


def _dense(P, J):
    rp, ci = P.graph()
    A = np.zeros((P.ndof, P.ndof))
    for i in range(P.ndof):
        A[i, ci[rp[i]:rp[i + 1]]] = J[rp[i]:rp[i + 1]]
    return A


@pytest.mark.parametrize("dim,order,kind", [(2, 1, "thermal"), (3, 1, "thermal"), (2, 2, "diffusion_1pu2"),
                                            (3, 1, "diffusion_1pu2"), (3, 2, "diffusion_1pu2")])
def test_ad_jacobian_matches_finite_differences(dim, order, kind):
    n = (3, 2, 2)[:dim] if order == 2 else (3, 3, 2)[:dim]
    rng = np.random.default_rng(7)
    ncell = int(np.prod(n))
    cfg = dict(dim=dim, order=order, n=n, kind=kind, source=("sinprod", 3.0, 2.0), kappa=np.exp(rng.standard_normal(ncell)),
               dirichlet_faces=1, vertex_coords=perturbed_vertices(dim, n, (0, 0, 0), (1, 1, 1), 0.2, 3))
    P = oracle_problem(cfg)
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
        col = -(rp_ - rm_) / (2 * eps)  # r = -res, J = d res / du
        np.testing.assert_allclose(A[free, j], col[free], rtol=1e-6, atol=1e-8 * np.abs(A).max())
    # Dirichlet rows: identity
    for d in fixed:
        assert A[d, d] == 1.0 and np.count_nonzero(A[d]) == 1


def _axis_range(i, N, p):
    ncell = (N - 1) // p
    cf, cl = ((i // p - 1, i // p) if i % p == 0 else (i // p, i // p))
    cf, cl = max(cf, 0), min(cl, ncell - 1)
    return p * cf, p * (cl - cf) + p + 1


@pytest.mark.parametrize("dim,order,n", [(2, 1, (5, 3)), (3, 1, (4, 3, 2)), (3, 2, (2, 3, 1)), (2, 2, (1, 4))])
def test_canonical_graph_layout_formula(dim, order, n):
    """The analytic per-axis layout used by the GPU kernels equals the oracle's union-of-couplings graph."""
    P = oracle_problem(dict(dim=dim, order=order, n=n))
    rp, ci = P.graph()
    NN = [order * v + 1 for v in n] + [1] * (3 - dim)
    pref, T = [], []
    for k in range(3):
        cnts = [(_axis_range(i, NN[k], order)[1] if k < dim else 1) for i in range(NN[k])]
        pref.append(np.concatenate([[0], np.cumsum(cnts)]))
        T.append(pref[k][-1])
    assert rp[-1] == T[0] * T[1] * T[2]
    for node in range(P.ndof):
        ix, iy, iz = node % NN[0], (node // NN[0]) % NN[1], node // (NN[0] * NN[1])
        cz = _axis_range(iz, NN[2], order)[1] if dim == 3 else 1
        cy = _axis_range(iy, NN[1], order)[1]
        expect = pref[2][iz] * T[1] * T[0] + cz * (pref[1][iy] * T[0] + cy * pref[0][ix])
        assert rp[node] == expect
        assert np.all(np.diff(ci[rp[node]:rp[node + 1]]) > 0)


def test_workset_size_and_threads_do_not_change_results():
    rng = np.random.default_rng(1)
    n = (6, 5, 4)
    kap = np.exp(0.5 * rng.standard_normal(int(np.prod(n))))
    base = dict(dim=3, order=1, n=n, kappa=kap, source=("sinprod", 2.0, 3.0), dirichlet_faces=3)
    u = rng.standard_normal((n[0] + 1) * (n[1] + 1) * (n[2] + 1))
    ref = oracle_problem(dict(base, workset_size=1)).assemble(u)
    for ws, th in [(100, 1), (7, 4), (1024, 2)]:
        r, J = oracle_problem(dict(base, workset_size=ws)).assemble(u, nthreads=th)
        np.testing.assert_allclose(r, ref[0], rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(J, ref[1], rtol=1e-13, atol=1e-15)
