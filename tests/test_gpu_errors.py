"""Failure handling through the C ABI; every failure is made on the host (no device fault)."""
import numpy as np
import pytest
import torch

from mrhyde_gb300 import _lib as L


@pytest.mark.gpu
def test_nan_kappa_rejected(cuda):
    from mrhyde_gb300 import Problem

    kap = np.ones(8)
    kap[3] = np.nan
    with pytest.raises(L.MrgError) as e:
        Problem(dim=3, order=1, n=(2, 2, 2), kappa=kap)
    assert e.value.status == L.MRG_ENUMERIC


@pytest.mark.gpu
def test_unsupported_modes_and_bad_buffers(cuda):
    from mrhyde_gb300 import AssemblyManager, Problem

    P = Problem(dim=2, order=1, n=(4, 4))
    A = AssemblyManager(P)
    u, r, J = P.new_vector(), P.new_vector(), P.new_matrix_values()
    with pytest.raises(L.MrgError) as e:
        A.assembleJacRes(u, r, J, is_adjoint=True)
    assert e.value.status == L.MRG_ENOTSUP
    with pytest.raises(L.MrgError) as e:
        A.assembleJacRes(u, r, J, compute_sens=True)
    assert e.value.status == L.MRG_ENOTSUP
    rc = L.lib().mrg_assemble(P.handle, torch.cuda.current_stream().cuda_stream and None, None, None, 3, None)
    assert rc == L.MRG_EINVAL
    with pytest.raises(ValueError):
        A.assembleJacRes(u[:-1], r, J)


@pytest.mark.gpu
def test_non_spd_matrix_reported_by_pcg(cuda):
    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager

    kap = -np.ones(16)  # negative definite operator: p.Jp < 0 at the first iteration
    P = Problem(dim=2, order=1, n=(4, 4), kappa=kap, dirichlet_faces=1)
    A, S = AssemblyManager(P), SolverManager(P)
    u, r, J = P.new_vector(), P.new_vector(), P.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x = P.new_vector()
    with pytest.raises(L.MrgError) as e:
        S.PCG(J, r, x, tol=1e-12, maxiter=200)
    assert e.value.status in (L.MRG_ENUMERIC, L.MRG_ENOCONV)
    # the context stays usable afterwards
    A.assembleJacRes(u, r, J, overwrite=True)
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_pcg_iteration_limit_reports_noconv(cuda):
    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager

    P = Problem(dim=3, order=1, n=(12, 12, 12), source=("const", 1.0, 0.0))
    A, S = AssemblyManager(P), SolverManager(P)
    u, r, J = P.new_vector(), P.new_vector(), P.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x = P.new_vector()
    res = S.PCG(J, r, x, tol=1e-14, maxiter=3, raise_on_noconv=False)
    assert res.iterations == 3
    with pytest.raises(L.MrgError) as e:
        S.PCG(J, r, P.new_vector(), tol=1e-14, maxiter=3)
    assert e.value.status == L.MRG_ENOCONV
